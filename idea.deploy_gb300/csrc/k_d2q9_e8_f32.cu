// D2Q9 + E8 kernels, FP32-shifted (BGK and MRT).
#include "launch.cuh"

namespace sclbm {
SCLBM_OPS_TU(ops_d2q9_e8_f32, D2Q9, D2E8, float, false)
}  // namespace sclbm
