// ints3c_lc4.cu — the 3-index integral and derivative class kernels with fitting shells of
// angular momentum 4.
#include "ints3c.cuh"

namespace gdfjk {
namespace ints {
Eri3Kernel pick_lc4(int la, int lb) { return pick_pair<4>(la, lb); }
Eri3GradKernel pick_grad_lc4(int la, int lb) { return pick_grad_pair<4>(la, lb); }
}  // namespace ints
}  // namespace gdfjk
