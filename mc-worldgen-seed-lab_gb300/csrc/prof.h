/* prof.h -- optional per-kernel CUDA-event timing of the library's own launches.
 *
 * When enabled (mcgen_gb300_profile), every launcher brackets its kernel with two events recorded on the
 * kernel's own stream, so a benchmark can divide a kernel's algorithmic work by its measured duration
 * inside the timed region.  Disabled, a launch costs one relaxed branch. */
#ifndef MG_PROF_H
#define MG_PROF_H
#include <cuda_runtime.h>

namespace mg {

enum {
    K_SETUP_XO = 0, K_SETUP_LEGACY, K_SETUP_END, K_POINTS, K_GRID, K_CHAIN_RESOLVE, K_BLOCKGRID, K_END_CHUNKS,
    K_END_LOOKUP, K_OW_SEED_CLIMATE, K_OW_FINISH_TREE, K_BATCH, K_SEARCH_CELLS, K_SEARCH_FIRST, K_SEARCH_REST,
    K_DENSITY, K_BATCH_EXACT, K_NUM_KERNELS
};
const char *kernel_name(int kid);
void prof_mark(int kid, cudaStream_t st, bool end);
int prof_enable(int on);
int prof_read(int kid, double *total_ms, long long *launches);

struct ProfScope {
    int kid;
    cudaStream_t st;
    ProfScope(int k, cudaStream_t s) : kid(k), st(s) { prof_mark(kid, st, false); }
    ~ProfScope() { prof_mark(kid, st, true); }
};

}  // namespace mg
#endif
