// D3Q19 + E6 kernels, FP32-shifted (BGK and MRT).
#include "launch.cuh"

namespace sclbm {
SCLBM_OPS_TU(ops_d3q19_e6_f32, D3Q19, D3E6, float, false)
}  // namespace sclbm
