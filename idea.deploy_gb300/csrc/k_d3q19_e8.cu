// D3Q19 + E8 instantiations (BGK, MRT; FP64, FP32-shifted).
#include "launch.cuh"

namespace sclbm {

const KernelOps *ops_d3q19_e8(bool mrt, bool fp32) {
    if (mrt) return fp32 ? Ops<D3Q19, D3E8, true, float>::ops() : Ops<D3Q19, D3E8, true, double>::ops();
    return fp32 ? Ops<D3Q19, D3E8, false, float>::ops() : Ops<D3Q19, D3E8, false, double>::ops();
}

}  // namespace sclbm
