// D2Q9 + E8 kernels, FP64, fused arithmetic (BGK and MRT).
#include "launch.cuh"

namespace sclbm {
SCLBM_OPS_TU(ops_d2q9_e8_f64, D2Q9, D2E8, double, false)
}  // namespace sclbm
