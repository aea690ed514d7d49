// D3Q19 + E4 instantiations (BGK, MRT; FP64, FP32-shifted).
#include "launch.cuh"

namespace sclbm {

const KernelOps *ops_d3q19_e4(bool mrt, bool fp32) {
    if (mrt) return fp32 ? Ops<D3Q19, D3E4, true, float>::ops() : Ops<D3Q19, D3E4, true, double>::ops();
    return fp32 ? Ops<D3Q19, D3E4, false, float>::ops() : Ops<D3Q19, D3E4, false, double>::ops();
}

}  // namespace sclbm
