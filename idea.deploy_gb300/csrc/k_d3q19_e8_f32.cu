// D3Q19 + E8 kernels, FP32-shifted (BGK and MRT).
#include "launch.cuh"

namespace sclbm {
SCLBM_OPS_TU(ops_d3q19_e8_f32, D3Q19, D3E8, float, false)
}  // namespace sclbm
