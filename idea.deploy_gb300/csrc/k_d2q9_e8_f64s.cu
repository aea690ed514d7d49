// D2Q9 + E8 kernels, FP64, reference arithmetic (BGK and MRT).
#include "launch.cuh"

namespace sclbm {
SCLBM_OPS_TU(ops_d2q9_e8_f64s, D2Q9, D2E8, double, true)
}  // namespace sclbm
