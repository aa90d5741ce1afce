/* noalloc.cu -- a seeds x points entry point that allocates no memory.
 *
 * mcgen_gb300_seed_points_dev keeps each seed's 46 noise lattices (14.7 KB per Overworld seed) in scratch
 * memory that it takes from the stream-ordered allocator on every call.  Some callers cannot let a library
 * allocate on their behalf: a runtime that owns every byte of device memory through its own arena, a
 * latency-critical loop that must never reach the driver's allocator, or an embedder that forbids
 * allocation once set-up is over.  For them this file keeps that scratch in one fixed, file-scope device
 * array and offers a variant entry point that uses it instead.
 *
 * The array is SEED_SCRATCH_BYTES (16 MiB) and lives in every GPU that loads the library until the process
 * exits.  Its device address is looked up once per device (cudaGetSymbolAddress) on the first call made
 * with that device current; make that first call before any stream capture.  Calls share the array and it
 * keeps the last call's lattices: each call overwrites every byte it reads, so nothing needs clearing, but
 * calls whose GPU work overlaps (different streams, no ordering between them) race on it.
 */
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/mcgen_gb300.h"
#include "abi_internal.h"
#include "launch.h"

#define SEED_SCRATCH_BYTES (16u << 20)
#define MAX_DEVICES 64

static __device__ __align__(256) unsigned char g_seed_scratch[SEED_SCRATCH_BYTES];
static void *g_seed_scratch_addr[MAX_DEVICES]; /* device address of g_seed_scratch, per device */

extern "C" MCGEN_API int mcgen_gb300_seed_points_noalloc(const McWorld *w, const int64_t *d_seeds, int ns,
                                                         const int32_t *d_qxyz, int np, uint8_t *d_out,
                                                         int32_t *d_targets, void *stream) {
    if (!w || ns < 0 || np < 0 || (ns > 0 && !d_seeds) || (np > 0 && (!d_qxyz || !d_out))) return MCGEN_E_ARG;
    if ((long long)ns * np == 0) return MCGEN_OK;
    if ((long long)ns * np > (1LL << 31)) return MCGEN_E_ARG;
    const size_t need = (size_t)ns * (size_t)w->desc.ntables * sizeof(MgLattice);
    if (need > SEED_SCRATCH_BYTES) return MCGEN_E_ARG; /* too many seeds for the fixed scratch: split the call */
    std::lock_guard<std::mutex> lk(mg::abi_lock());
    if (!w->dev_ready) return MCGEN_E_ARG; /* the world is not on the device yet: any earlier biome call puts it there */
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= MAX_DEVICES) return MCGEN_E_INTERNAL;
    if (dev != mg::abi_device()) return MCGEN_E_ARG; /* the world's data lives on the library's device */
    if (!g_seed_scratch_addr[dev]) {
        void *p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_seed_scratch);
        if (e != cudaSuccess) return mg::abi_cuda_code((int)e);
        if (!p) return MCGEN_E_INTERNAL;
        g_seed_scratch_addr[dev] = p;
    }
    MgLattice *states = (MgLattice *)g_seed_scratch_addr[dev];
    cudaStream_t st = (cudaStream_t)stream;
    int rc = mg::launch_setup(w->desc, d_seeds, ns, states, st);
    if (!rc) rc = mg::launch_points(w->desc, w->d_tree, states, ns, d_qxyz, np, d_out, d_targets, st);
    /* a launch error is reported as mcgen_gb300_seed_points_dev reports it */
    return mg::abi_cuda_code(rc);
}
