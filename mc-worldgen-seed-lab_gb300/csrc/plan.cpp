/* plan.cpp -- the batched form's host side: McGb300Plan (mcgen_gb300_plan_*).
 *
 * A plan freezes a list of requests: it uploads the distinct worlds (descriptions and R-tree pointers),
 * assigns every distinct (world, seed) a slot in a lattice pool, numbers the tiles of every request
 * (batch.cu), and lays the outputs out back to back.  Running it enqueues the per-seed setup launches (one
 * per dimension present) and the persistent k_batch launch.  The first run on a stream captures those
 * launches into a CUDA graph on a private stream and later runs replay it; the tile shape is chosen by
 * timing the four shapes on the plan itself (mcgen_gb300_plan_autotune).
 */
#include <cuda_runtime.h>
#include <string.h>

#include <algorithm>
#include <map>
#include <unordered_map>
#include <mutex>
#include <vector>

#include "../../include/mcgen_gb300.h"
#include "abi_internal.h"
#include "batch.h"
#include "launch.h"

struct McGb300Plan {
    int nreq = 0;
    long long ntiles[BATCH_SHAPES] = {0, 0, 0, 0};
    long long out_bytes = 0;
    long long h2d_bytes = 0; /* bytes copied to the device by plan_new */
    std::vector<long long> out_off;
    std::vector<long long> cells;
    int shape = 0;
    int ctas = 0;
    /* device: one allocation (d_arena) holds the lists, the lattice pool and the tile counter */
    void *d_arena = nullptr;
    MgWorldDesc *d_worlds = nullptr;
    const MgTreeNode **d_trees = nullptr;
    MgBatchReq *d_reqs[BATCH_SHAPES] = {nullptr, nullptr, nullptr, nullptr};
    MgSetupEntry *d_ent[3] = {nullptr, nullptr, nullptr};
    int nent[3] = {0, 0, 0};
    int *d_first = nullptr; /* Overworld: first lattice of each entry, relative to the Overworld list */
    long long ow_lattices = 0;
    MgLattice *d_pool = nullptr;
    unsigned long long *d_counter = nullptr; /* tiles taken, cells recorded for the exact pass */
    MgPending *d_pend = nullptr;             /* records of double-branch Overworld cells left to the exact pass */
    long long pend_cap = 0;
    /* graph of one run */
    cudaStream_t cap = nullptr;
    cudaGraphExec_t exec = nullptr;
    uint8_t *graph_out = nullptr;
    int graph_shape = -1;
    /* completion of the latest run: runs share the lattice pool and the tile counter, so each run waits for
     * the previous one whatever stream it is on, and freeing the plan waits for the last in stream order */
    cudaEvent_t last_run = nullptr;
    bool ran = false;
    std::vector<McWorld *> held; /* worlds kept alive while the plan exists */
};

namespace {

/* hash of a (world index, seed) key */
struct SeedKeyHash {
    size_t operator()(const std::pair<int, int64_t> &k) const {
        uint64_t x = (uint64_t)k.second * 0x9E3779B97F4A7C15ULL ^ (uint64_t)(uint32_t)k.first * 0xC2B2AE3D27D4EB4FULL;
        return (size_t)(x ^ (x >> 31));
    }
};

int cuda_rc(cudaError_t e) { return e == cudaSuccess ? MCGEN_OK : e == cudaErrorMemoryAllocation ? MCGEN_E_NOMEM : MCGEN_E_INTERNAL; }

/* Device memory of plans and of the host-buffer run's output: a stream-ordered pool of the library's that
 * keeps up to 4 GiB of freed memory mapped for the next plan (the device's default pool returns it at every
 * synchronisation, and a plan's arena plus a run's output are hundreds of MB: mapping them again each time
 * cost milliseconds per call).  Created on first use, under the ABI lock. */
cudaMemPool_t g_pool = nullptr;
int g_pool_dev = -1;
cudaError_t plan_pool(cudaMemPool_t *out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e) return e;
    if (!g_pool || g_pool_dev != dev) {
        cudaMemPoolProps props;
        memset(&props, 0, sizeof props);
        props.allocType = cudaMemAllocationTypePinned;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = dev;
        cudaMemPool_t pool = nullptr;
        if ((e = cudaMemPoolCreate(&pool, &props))) return e;
        uint64_t keep = 4ULL << 30;
        if ((e = cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep))) {
            cudaMemPoolDestroy(pool);
            return e;
        }
        g_pool = pool; /* a pool of another device stays alive: memory of plans made there returns to it */
        g_pool_dev = dev;
    }
    *out = g_pool;
    return cudaSuccess;
}

int enqueue(McGb300Plan *p, uint8_t *d_out, int shape, cudaStream_t st) {
    for (int d = 0; d < 3; d++) {
        if (!p->nent[d]) continue;
        int rc = mg::launch_setup_list(p->d_worlds, d, p->d_ent[d], p->nent[d], p->d_first, p->ow_lattices, p->d_pool, st);
        if (rc) return rc;
    }
    return mg::launch_batch(p->d_worlds, p->d_trees, p->d_reqs[shape], p->nreq, p->ntiles[shape], p->d_pool,
                            p->d_counter, p->d_pend, p->pend_cap, d_out, p->ctas, shape, st);
}

/* Order a run on `st` after the plan's previous run (on any stream); caller holds the ABI lock. */
int run_begin(McGb300Plan *p, cudaStream_t st) {
    if (!p->ran) return MCGEN_OK;
    return cuda_rc(cudaStreamWaitEvent(st, p->last_run, 0));
}
int run_end(McGb300Plan *p, cudaStream_t st) {
    cudaError_t e = cudaEventRecord(p->last_run, st);
    if (!e) p->ran = true;
    return cuda_rc(e);
}

/* Caller holds the ABI lock.  Nothing here blocks the host: a graph or stream still in use is released by
 * the driver when its work completes, and the arena returns to the pool after the last run. */
void free_plan(McGb300Plan *p) {
    if (p->exec) cudaGraphExecDestroy(p->exec);
    if (p->cap) cudaStreamDestroy(p->cap);
    if (p->d_arena) {
        cudaStream_t ast = mg::abi_stream();
        if (p->ran) cudaStreamWaitEvent(ast, p->last_run, 0);
        cudaFreeAsync(p->d_arena, ast);
    }
    if (p->last_run) cudaEventDestroy(p->last_run);
    for (McWorld *w : p->held) mg::abi_world_release(w);
    delete p;
}

}  // namespace

extern "C" {

MCGEN_API int mcgen_gb300_plan_new(const McGb300Request *reqs, int n, int tie_rule, McGb300Plan **out) {
    if (!out || n < 0 || (n > 0 && !reqs)) return MCGEN_E_ARG;
    if (tie_rule != MCGEN_TIE_ENGINE && tie_rule != MCGEN_TIE_CHUNK_CELL) return MCGEN_E_ARG;
    *out = nullptr;
    for (int i = 0; i < n; i++) {
        const McGb300Request &r = reqs[i];
        if (!r.world || r.nx <= 0 || r.nz <= 0 || (long long)r.nx * r.nz > (1LL << 31)) return MCGEN_E_ARG;
        if ((long long)r.qx0 + r.nx > INT32_MAX || (long long)r.qz0 + r.nz > INT32_MAX) return MCGEN_E_ARG;
    }
    std::lock_guard<std::mutex> lk(mg::abi_lock());
    if (!mg::abi_device_ready()) return MCGEN_E_UNSUPPORTED;
    McGb300Plan *p = new McGb300Plan();
    p->nreq = n;
    /* distinct worlds; each must have its device copy (tree) */
    std::map<const McWorld *, int> widx;
    std::vector<const McWorld *> worlds;
    std::vector<int> wof((size_t)n); /* world index of each request */
    for (int i = 0; i < n; i++) {
        auto it = widx.find(reqs[i].world);
        if (it == widx.end()) it = widx.emplace(reqs[i].world, (int)worlds.size()).first, worlds.push_back(reqs[i].world);
        wof[(size_t)i] = it->second;
    }
    for (auto *w : worlds) {
        int rc = mg::abi_world_device(const_cast<McWorld *>(w));
        if (rc) { free_plan(p); return rc; }
        mg::abi_world_hold(const_cast<McWorld *>(w));
        p->held.push_back(const_cast<McWorld *>(w));
    }
    if (cudaError_t ee = cudaEventCreateWithFlags(&p->last_run, cudaEventDisableTiming)) {
        p->last_run = nullptr;
        free_plan(p);
        return cuda_rc(ee);
    }
    /* distinct (world, seed) -> pool slots, grouped by dimension (a hashed map: an ordered one cost most of a
     * 10,000-request plan's host time; slots follow the requests' first occurrences either way) */
    std::unordered_map<std::pair<int, int64_t>, int, SeedKeyHash> slot_of;
    slot_of.reserve((size_t)n * 2);
    std::vector<int> slot((size_t)n); /* pool slot of each request */
    std::vector<MgSetupEntry> ent[3];
    std::vector<int> first;
    long long pool = 0, ow = 0;
    for (int i = 0; i < n; i++) {
        const int wi = wof[(size_t)i];
        auto ins = slot_of.emplace(std::make_pair(wi, (int64_t)reqs[i].seed), (int)pool);
        slot[(size_t)i] = ins.first->second;
        if (!ins.second) continue;
        const MgWorldDesc &W = worlds[(size_t)wi]->desc;
        MgSetupEntry e;
        e.seed = reqs[i].seed;
        e.world = wi;
        e.slot = (int32_t)pool;
        if (W.dim == MG_OVERWORLD) { first.push_back((int)ow); ow += W.ntables; }
        ent[W.dim].push_back(e);
        pool += W.ntables;
        if (pool > INT32_MAX) { free_plan(p); return MCGEN_E_ARG; }
    }
    p->ow_lattices = ow;
    /* requests and tiles for every shape; outputs back to back */
    std::vector<MgBatchReq> rq[BATCH_SHAPES];
    for (auto &v : rq) v.reserve((size_t)n);
    p->out_off.resize((size_t)n);
    p->cells.resize((size_t)n);
    long long off = 0;
    for (int i = 0; i < n; i++) {
        p->out_off[(size_t)i] = off;
        p->cells[(size_t)i] = (long long)reqs[i].nx * reqs[i].nz;
        off += p->cells[(size_t)i];
    }
    p->out_bytes = off;
    long long dcells = 0; /* double-branch Overworld cells: the ones the exact pass may take */
    for (int i = 0; i < n; i++) {
        const MgWorldDesc &W = worlds[(size_t)wof[(size_t)i]]->desc;
        if (W.dim == MG_OVERWORLD && !W.fmode) dcells += p->cells[(size_t)i];
    }
    p->pend_cap = tie_rule == MCGEN_TIE_ENGINE ? mg::batch_pending_cap(dcells) : 0;
    /* processing order: requests grouped by world, heaviest code path first (Overworld double branch, then
     * float, Nether, End), so that the CTAs resident at any time run the same code (the kernel holds every
     * dimension and branch; mixing them thrashes the instruction cache) and the light tiles come last */
    std::vector<int> order((size_t)n);
    for (int i = 0; i < n; i++) order[(size_t)i] = i;
    std::vector<int> key((size_t)n); /* code path, then world */
    for (int i = 0; i < n; i++) {
        const MgWorldDesc &W = worlds[(size_t)wof[(size_t)i]]->desc;
        key[(size_t)i] = (W.dim * 2 + (W.fmode ? 1 : 0)) * (int)(worlds.size() + 1) + wof[(size_t)i];
    }
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return key[(size_t)a] < key[(size_t)b]; });
    for (int s = 0; s < BATCH_SHAPES; s++) {
        long long tiles = 0;
        for (int i : order) {
            const McGb300Request &r = reqs[i];
            const int wi = wof[(size_t)i];
            MgBatchReq b;
            b.world = wi;
            b.state = slot[(size_t)i];
            b.qx0 = r.qx0; b.qz0 = r.qz0; b.nx = r.nx; b.nz = r.nz; b.qy = r.qy;
            b.tie = worlds[(size_t)wi]->desc.dim == MG_END ? MG_TIE_ENGINE : tie_rule;
            b.tile0 = tiles;
            b.out_off = p->out_off[(size_t)i];
            tiles += mg::batch_tiles(worlds[(size_t)wi]->desc.dim, r.qx0, r.qz0, r.nx, r.nz, s);
            rq[s].push_back(b);
        }
        p->ntiles[s] = tiles;
    }
    /* device copies: the lists are staged back to back (256-byte aligned) and uploaded in one copy; the
     * lattice pool and the tile counter follow them in the same allocation */
    std::vector<MgWorldDesc> wd;
    std::vector<const MgTreeNode *> tp;
    for (auto *w : worlds) { wd.push_back(w->desc); tp.push_back(w->d_tree); }
    struct Part { void **dst; const void *src; size_t bytes, off; };
    std::vector<Part> parts;
    size_t at = 0;
    auto place = [&](void **dst, const void *src, size_t bytes) {
        if (!bytes) return;
        at = (at + 255) & ~(size_t)255;
        parts.push_back({dst, src, bytes, at});
        at += bytes;
    };
    place((void **)&p->d_worlds, wd.data(), sizeof(MgWorldDesc) * wd.size());
    place((void **)&p->d_trees, tp.data(), sizeof(void *) * tp.size());
    for (int s = 0; s < BATCH_SHAPES; s++) place((void **)&p->d_reqs[s], rq[s].data(), sizeof(MgBatchReq) * rq[s].size());
    for (int d = 0; d < 3; d++) {
        p->nent[d] = (int)ent[d].size();
        place((void **)&p->d_ent[d], ent[d].data(), sizeof(MgSetupEntry) * ent[d].size());
    }
    place((void **)&p->d_first, first.data(), sizeof(int) * first.size());
    const size_t staged = at;
    std::vector<uint8_t> host(staged);
    for (const Part &q : parts) memcpy(host.data() + q.off, q.src, q.bytes);
    const size_t pool_off = (at + 255) & ~(size_t)255;
    const size_t counter_off = pool_off + sizeof(MgLattice) * (size_t)pool;
    const size_t pend_off = counter_off + 2 * sizeof(unsigned long long);
    const size_t arena_bytes = pend_off + sizeof(MgPending) * (size_t)p->pend_cap;
    cudaMemPool_t mp = nullptr;
    cudaStream_t ast = mg::abi_stream();
    cudaError_t e = plan_pool(&mp);
    if (!e) e = cudaMallocFromPoolAsync(&p->d_arena, arena_bytes, mp, ast);
    if (!e && staged) e = cudaMemcpyAsync(p->d_arena, host.data(), staged, cudaMemcpyHostToDevice, ast);
    if (!e) e = cudaStreamSynchronize(ast); /* the arena is ready for any stream */
    if (!e) {
        uint8_t *base = (uint8_t *)p->d_arena;
        for (const Part &q : parts) *q.dst = base + q.off;
        if (pool) p->d_pool = (MgLattice *)(base + pool_off);
        p->d_counter = (unsigned long long *)(base + counter_off);
        if (p->pend_cap) p->d_pend = (MgPending *)(base + pend_off);
        p->h2d_bytes = (long long)staged;
    }
    if (!e) e = (cudaError_t)mg::batch_prepare(nullptr);
    if (e) {
        free_plan(p);
        return cuda_rc(e);
    }
    p->ctas = 0; /* each tile shape runs its own resident grid */
    *out = p;
    return MCGEN_OK;
}

MCGEN_API void mcgen_gb300_plan_free(McGb300Plan *p) {
    if (!p) return;
    std::lock_guard<std::mutex> lk(mg::abi_lock());
    free_plan(p);
}

MCGEN_API long long mcgen_gb300_plan_output_bytes(const McGb300Plan *p) { return p ? p->out_bytes : -1; }
MCGEN_API long long mcgen_gb300_plan_output_offset(const McGb300Plan *p, int i) {
    return (p && i >= 0 && i < p->nreq) ? p->out_off[(size_t)i] : -1;
}
MCGEN_API int mcgen_gb300_plan_shape(const McGb300Plan *p) { return p ? p->shape : -1; }
MCGEN_API long long mcgen_gb300_plan_h2d_bytes(const McGb300Plan *p) { return p ? p->h2d_bytes : -1; }
MCGEN_API int mcgen_gb300_plan_set_shape(McGb300Plan *p, int shape) {
    if (!p || shape < 0 || shape >= BATCH_SHAPES) return MCGEN_E_ARG;
    p->shape = shape;
    return MCGEN_OK;
}

/* Run into device memory (plan_output_bytes bytes at d_out) on `stream`, through the plan's CUDA graph. */
MCGEN_API int mcgen_gb300_plan_run_dev(McGb300Plan *p, uint8_t *d_out, void *stream) {
    if (!p || (!d_out && p->out_bytes)) return MCGEN_E_ARG;
    if (!p->nreq) return MCGEN_OK;
    std::lock_guard<std::mutex> lk(mg::abi_lock());
    cudaStream_t st = (cudaStream_t)stream;
    cudaError_t e;
    if (!p->exec || p->graph_out != d_out || p->graph_shape != p->shape) {
        if (p->exec) { cudaGraphExecDestroy(p->exec); p->exec = nullptr; }
        if (!p->cap && (e = cudaStreamCreateWithFlags(&p->cap, cudaStreamNonBlocking))) return cuda_rc(e);
        if ((e = cudaStreamBeginCapture(p->cap, cudaStreamCaptureModeThreadLocal))) return cuda_rc(e);
        int rc = enqueue(p, d_out, p->shape, p->cap);
        cudaGraph_t g = nullptr;
        e = cudaStreamEndCapture(p->cap, &g);
        if (rc || e) { if (g) cudaGraphDestroy(g); return rc ? MCGEN_E_INTERNAL : cuda_rc(e); }
        e = cudaGraphInstantiate(&p->exec, g, 0);
        cudaGraphDestroy(g);
        if (e) { p->exec = nullptr; return cuda_rc(e); }
        p->graph_out = d_out;
        p->graph_shape = p->shape;
    }
    int rc = run_begin(p, st);
    if (!rc) rc = cuda_rc(cudaGraphLaunch(p->exec, st));
    if (!rc) rc = run_end(p, st);
    return rc;
}

/* The same without a graph (each launch visible to the library's per-kernel profiler). */
MCGEN_API int mcgen_gb300_plan_run_dev_direct(McGb300Plan *p, uint8_t *d_out, void *stream) {
    if (!p || (!d_out && p->out_bytes)) return MCGEN_E_ARG;
    std::lock_guard<std::mutex> lk(mg::abi_lock());
    cudaStream_t st = (cudaStream_t)stream;
    int rc = run_begin(p, st);
    if (rc) return rc;
    if (enqueue(p, d_out, p->shape, st)) return MCGEN_E_INTERNAL;
    return run_end(p, st);
}

/* Time every tile shape on the plan itself (reps runs each, after one warm-up) and keep the fastest.
 * d_out: a device buffer of plan_output_bytes. */
MCGEN_API int mcgen_gb300_plan_autotune(McGb300Plan *p, uint8_t *d_out, int reps, double *best_ms) {
    if (!p || (!d_out && p->out_bytes) || reps <= 0) return MCGEN_E_ARG;
    std::lock_guard<std::mutex> lk(mg::abi_lock());
    cudaStream_t st;
    if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking)) return MCGEN_E_INTERNAL;
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    double best = 1e30;
    int best_s = 0, rc = run_begin(p, st);
    for (int s = 0; s < BATCH_SHAPES && !rc; s++) {
        rc = enqueue(p, d_out, s, st);
        cudaEventRecord(a, st);
        for (int r = 0; r < reps && !rc; r++) rc = enqueue(p, d_out, s, st);
        cudaEventRecord(b, st);
        if (cudaEventSynchronize(b)) rc = MCGEN_E_INTERNAL;
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, a, b);
        if (!rc && ms / reps < best) { best = ms / reps; best_s = s; }
    }
    if (!rc) rc = run_end(p, st);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    cudaStreamDestroy(st);
    if (rc) return MCGEN_E_INTERNAL;
    p->shape = best_s;
    if (best_ms) *best_ms = best;
    return MCGEN_OK;
}

/* Host-buffer form: runs the plan (direct launches: a one-off run gains nothing from a graph) and copies
 * the outputs to `out` (plan_output_bytes bytes). */
MCGEN_API int mcgen_gb300_plan_run(McGb300Plan *p, uint8_t *out) {
    if (!p || (!out && p->out_bytes)) return MCGEN_E_ARG;
    if (!p->nreq) return MCGEN_OK;
    uint8_t *d_out = nullptr;
    cudaStream_t st = mg::abi_stream();
    cudaMemPool_t mp = nullptr;
    cudaError_t e;
    {
        std::lock_guard<std::mutex> lk(mg::abi_lock());
        e = plan_pool(&mp);
    }
    if (!e) e = cudaMallocFromPoolAsync((void **)&d_out, (size_t)p->out_bytes, mp, st);
    if (e) return cuda_rc(e);
    int rc = mcgen_gb300_plan_run_dev_direct(p, d_out, st);
    if (!rc) rc = cuda_rc(cudaMemcpyAsync(out, d_out, (size_t)p->out_bytes, cudaMemcpyDeviceToHost, st));
    cudaFreeAsync(d_out, st);
    cudaError_t e2 = cudaStreamSynchronize(st);
    return rc ? rc : cuda_rc(e2);
}

}  // extern "C"
