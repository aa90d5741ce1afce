/* batch.h -- device layouts and launchers of the batched (many requests, one launch) form. */
#ifndef MG_BATCH_H
#define MG_BATCH_H
#include <cuda_runtime.h>
#include <stdint.h>

#include "mg_types.h"

/* one request of a batch: a quart-resolution region of one (world, seed) */
typedef struct {
    int32_t world;   /* index into the batch's world table */
    int32_t state;   /* first lattice of its seed in the state pool */
    int32_t qx0, qz0, nx, nz, qy;
    int32_t tie;     /* MG_TIE_ENGINE or MG_TIE_CHUNK_CELL */
    int64_t tile0;   /* number of the request's first tile */
    int64_t out_off; /* its first output byte */
} MgBatchReq;

/* one (world, seed) whose lattices the setup kernels write at pool[slot ...] */
typedef struct {
    int64_t seed;
    int32_t world;
    int32_t slot;
} MgSetupEntry;

#define BATCH_SHAPES 4
namespace mg {
/* records to provide for a batch with `cells` double-branch Overworld cells (a bound far above the
 * measured 1.5-3.5e-4 share of unsettled values; cells beyond it take the exact path in place) */
long long batch_pending_cap(long long cells);
/* tile widths of the four Overworld/Nether tile shapes (128 cells each; the shapes also differ in the
 * register budget: 9, 7, 6 and 8 resident CTAs per SM) */
extern const int kBatchTileWidths[BATCH_SHAPES];
/* tiles of a request: 128 quart cells of shape `shape` (Overworld, Nether) or 8 x 8 chunks (End) */
long long batch_tiles(int dim, int qx0, int qz0, int nx, int nz, int shape);
/* lattices of a list of entries of one dimension; Overworld needs the prefix sums of lattices per entry */
int launch_setup_list(const MgWorldDesc *d_worlds, int dim, const MgSetupEntry *d_ent, int n, const int *d_first,
                      long long total_lattices, MgLattice *d_pool, cudaStream_t st);
/* kernel attributes and resident grid sizes; call before any stream capture */
int batch_prepare(int *ctas_per_sm);
/* ctas: upper bound on the persistent grid, 0 = every resident CTA of the shape.  d_counter holds two
 * counters (tiles taken, cells recorded); with d_pend (pend_cap records) the double-branch Overworld cells
 * left to the exact evaluation are recorded and finished by a second launch, without it in place. */
int launch_batch(const MgWorldDesc *d_worlds, const MgTreeNode *const *d_trees, const MgBatchReq *d_reqs, int nreq,
                 long long ntiles, const MgLattice *d_pool, unsigned long long *d_counter, MgPending *d_pend,
                 long long pend_cap, uint8_t *d_out, int ctas, int shape, cudaStream_t st);
}  // namespace mg
#endif
