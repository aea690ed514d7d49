// D2Q9 instantiations (E4, E6, E8; BGK, MRT; FP64, FP32-shifted).
#include "launch.cuh"

namespace sclbm {

template <class S>
static const KernelOps *pick(bool mrt, bool fp32) {
    if (mrt) return fp32 ? Ops<D2Q9, S, true, float>::ops() : Ops<D2Q9, S, true, double>::ops();
    return fp32 ? Ops<D2Q9, S, false, float>::ops() : Ops<D2Q9, S, false, double>::ops();
}

const KernelOps *ops_d2q9(int order, bool mrt, bool fp32) {
    switch (order) {
    case 4: return pick<D2E4>(mrt, fp32);
    case 6: return pick<D2E6>(mrt, fp32);
    case 8: return pick<D2E8>(mrt, fp32);
    default: return nullptr;
    }
}

}  // namespace sclbm
