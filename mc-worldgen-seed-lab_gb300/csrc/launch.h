/* launch.h -- host launchers of the biome kernels (kernels.cu), called by the C ABI (api.cpp).
 * All return a cudaError_t value (0 on success) and enqueue on `st` without synchronising. */
#ifndef MG_LAUNCH_H
#define MG_LAUNCH_H
#include <cuda_runtime.h>
#include <stddef.h>

#include "mg_types.h"

namespace mg {

long long launch_count();
void count_launch_external(); /* for launchers outside kernels.cu */

/* per-seed lattices: d_states[s * W.ntables + j] */
int launch_setup(const MgWorldDesc &W, const int64_t *d_seeds, int ns, MgLattice *d_states, cudaStream_t st);

/* seeds x quart points, ENGINE rule (targets optional) */
int launch_points(const MgWorldDesc &W, const MgTreeNode *tree, const MgLattice *states, int ns, const int32_t *pts,
                  int np, uint8_t *out, int32_t *targets, cudaStream_t st);

/* seeds x points for the Overworld (fused.cu): lattices built and sampled in shared memory by one kernel,
 * climate finish + R-tree by a second.  Scratch: fused_scratch_bytes(W, ns * np) (five noise values per
 * sample).  fused_supported() tells whether a world's lattice count fits the kernel. */
bool fused_supported(const MgWorldDesc &W);
size_t fused_scratch_bytes(const MgWorldDesc &W, long long samples);
int launch_ow_seed_points(const MgWorldDesc &W, const MgTreeNode *tree, const int64_t *seeds, int ns, const int32_t *pts,
                          int np, uint8_t *out, int32_t *targets, void *scratch, cudaStream_t st);

/* seed search, Overworld, first observation (one quart cell per candidate at pts[3i..3i+2]): candidates
 * that pass go to surv (count *nsurv), failures are added to *fail.  Scratch: fused_scratch_bytes(W, ns). */
int launch_ow_search_first(const MgWorldDesc &W, const MgTreeNode *tree, const int64_t *seeds, int ns, const int32_t *pts,
                           const MgObs &o, int ties, void *scratch, int64_t *surv, unsigned *nsurv,
                           unsigned long long *fail, cudaStream_t st);

/* one seed's quart grid.  Scratch: chain_scratch_bytes(nx*nz) for GRID_CHAIN and CHUNK_ORDER; for the End,
 * (nx/4 + 2) * (nz/4 + 2) bytes of chunk classes. */
size_t chain_scratch_bytes(long long ncells);
int launch_quart_grid(const MgWorldDesc &W, const MgTreeNode *tree, const MgLattice *state, int qx0, int qz0, int nx,
                      int nz, int qy, int rule, uint8_t *out, void *scratch, cudaStream_t st);

/* block-coordinate biomes (zoom + chunk-cell ties): a grid when xyz == nullptr, else nx points at xyz
 * (nz == 1).  End: scratch = chunk classes of [ecx0, ecx0+encx) x [ecz0, ecz0+encz), or null to evaluate
 * the class per sample. */
int launch_block_biomes(const MgWorldDesc &W, const MgTreeNode *tree, const MgLattice *state, int64_t zseed, int x0,
                        int z0, int nx, int nz, int step, int y, const int32_t *xyz, uint8_t *out, void *scratch,
                        int ecx0, int ecz0, int encx, int encz, cudaStream_t st);

/* Overworld density functions (continents, erosion, ridges, offset, depth) at n block points xyz[3i..3i+2] of
 * one seed's lattices: out[5i + k] (cudaErrorInvalidValue for other dimensions) */
int launch_density(const MgWorldDesc &W, const MgLattice *state, int n, const int32_t *xyz, double *out, cudaStream_t st);

/* pipe microbenchmarks (pipes.cu) */
int pipe_rate(int pipe, double *gops);

}  // namespace mg
#endif
