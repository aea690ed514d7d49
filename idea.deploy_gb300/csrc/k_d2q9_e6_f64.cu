// D2Q9 + E6 kernels, FP64, fused arithmetic (BGK and MRT).
#include "launch.cuh"

namespace sclbm {
SCLBM_OPS_TU(ops_d2q9_e6_f64, D2Q9, D2E6, double, false)
}  // namespace sclbm
