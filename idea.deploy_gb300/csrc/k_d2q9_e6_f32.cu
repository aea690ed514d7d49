// D2Q9 + E6 kernels, FP32-shifted (BGK and MRT).
#include "launch.cuh"

namespace sclbm {
SCLBM_OPS_TU(ops_d2q9_e6_f32, D2Q9, D2E6, float, false)
}  // namespace sclbm
