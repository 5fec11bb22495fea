// k_mixed.cu — split-precision exchange path (placeholder until the tcgen05 kernels land).
#include "gdfjk.h"
#include "mixed.cuh"

namespace gdfjk {

struct MixedState {
    int dummy = 0;
};

MixedState* mixed_create() { return new MixedState(); }
void mixed_destroy(MixedState* m) { delete m; }
void mixed_invalidate(MixedState*) {}
size_t mixed_query_memory(int, int, int) { return 0; }
int mixed_build_K(MixedState*, const double*, const TileLayout&, int, int, int, const double*, int, int, int, double*,
                  cudaEvent_t, cudaStream_t, std::string& err) {
    err = "mixed-precision K is not available in this build";
    return GDFJK_ERR_ARG;
}

}  // namespace gdfjk
