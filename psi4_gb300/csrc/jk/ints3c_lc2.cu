// ints3c_lc2.cu — the 3-index integral and derivative class kernels with fitting shells of
// angular momentum 2.
#include "ints3c.cuh"

namespace gdfjk {
namespace ints {
Eri3Kernel pick_lc2(int la, int lb) { return pick_pair<2>(la, lb); }
Eri3GradKernel pick_grad_lc2(int la, int lb) { return pick_grad_pair<2>(la, lb); }
}  // namespace ints
}  // namespace gdfjk
