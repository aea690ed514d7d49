// D3Q19 + E8 kernels, FP64, reference arithmetic (BGK and MRT).
#include "launch.cuh"

namespace sclbm {
SCLBM_OPS_TU(ops_d3q19_e8_f64s, D3Q19, D3E8, double, true)
}  // namespace sclbm
