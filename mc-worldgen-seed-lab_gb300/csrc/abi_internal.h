/* abi_internal.h -- the opaque handles of the C ABI, shared by the translation units that implement it. */
#ifndef MG_ABI_INTERNAL_H
#define MG_ABI_INTERNAL_H
#include <mutex>
#include <string>
#include <vector>

#include "../../include/mcgen.h"
#include "mg_types.h"

struct McGen {
    int version;
    std::string root;
};

struct McWorld {
    McGen *g;
    int dim;
    std::string preset;
    McSeeds seeds;
    int64_t zoom_seed;
    MgWorldDesc desc;
    std::vector<MgTreeNode> tree;
    /* device copies, created on first GPU use */
    int dev_ready;
    MgTreeNode *d_tree;
    MgLattice *d_state;
    /* identity that no other world of the process ever has (caches key on it, never on the address) */
    uint64_t uid;
    /* plans and pending served requests that use the world (under the ABI lock); mcgen_world_free while
     * holds > 0 only marks it, and the last release frees it */
    int holds;
    int free_requested;
};

#include <cuda_runtime.h>

namespace mg {
std::mutex &abi_lock(); /* serialises GPU work of all entry points */
int abi_device();       /* the device the library runs on */
/* with abi_lock held: select and initialise the device (1 = ready), give the library's stream, put a
 * world's tree and seed lattices on the device (MCGEN_OK or an error code) */
int abi_device_ready();
cudaStream_t abi_stream();
int abi_world_device(McWorld *w);
/* with abi_lock held: take / drop a reference that keeps a world (its description and device tree) alive
 * past mcgen_world_free until the last reference is dropped */
void abi_world_hold(McWorld *w);
void abi_world_release(McWorld *w);
/* a CUDA error code as the ABI reports it (MCGEN_E_NOMEM for an allocation failure, else MCGEN_E_INTERNAL;
 * the text goes to mcgen_gb300_last_error), MCGEN_OK for cudaSuccess */
int abi_cuda_code(int e);
}  // namespace mg
#endif
