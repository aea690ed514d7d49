// D3Q19 + E8 kernels, FP64, fused arithmetic (BGK and MRT).
#include "launch.cuh"

namespace sclbm {
SCLBM_OPS_TU(ops_d3q19_e8_f64, D3Q19, D3E8, double, false)
}  // namespace sclbm
