// ints3c_lc1.cu — the 3-index integral and derivative class kernels with fitting shells of
// angular momentum 1.
#include "ints3c.cuh"

namespace gdfjk {
namespace ints {
Eri3Kernel pick_lc1(int la, int lb) { return pick_pair<1>(la, lb); }
Eri3GradKernel pick_grad_lc1(int la, int lb) { return pick_grad_pair<1>(la, lb); }
}  // namespace ints
}  // namespace gdfjk
