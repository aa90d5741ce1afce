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
}  // namespace mg
#endif
