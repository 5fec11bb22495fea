// ints3c_lc0.cu — the 3-index integral and derivative class kernels with fitting shells of
// angular momentum 0.
#include "ints3c.cuh"

namespace gdfjk {
namespace ints {
Eri3Kernel pick_lc0(int la, int lb) { return pick_pair<0>(la, lb); }
Eri3GradKernel pick_grad_lc0(int la, int lb) { return pick_grad_pair<0>(la, lb); }
}  // namespace ints
}  // namespace gdfjk
