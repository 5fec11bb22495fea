// ints3c_lc3.cu — the 3-index integral and derivative class kernels with fitting shells of
// angular momentum 3.
#include "ints3c.cuh"

namespace gdfjk {
namespace ints {
Eri3Kernel pick_lc3(int la, int lb) { return pick_pair<3>(la, lb); }
Eri3GradKernel pick_grad_lc3(int la, int lb) { return pick_grad_pair<3>(la, lb); }
}  // namespace ints
}  // namespace gdfjk
