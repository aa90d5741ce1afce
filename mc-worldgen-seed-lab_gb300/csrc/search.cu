/* search.cu -- the biome seed search: which candidate seeds produce the observed biomes
 * (crack/src/gpu_biomes/gpu_biomes.cu:36-52 k_search, :199-243 search_gpu_impl; per-seed checks
 * engine/cuda/mc_gpu.cuh:476-493, 552-561, 685-693).
 *
 * Candidates come from a list, a structure seed (base | i << 48, i < 2^16) or a range (base + i), in chunks.
 * Overworld: every candidate's lattices are built and sampled at its first observation in shared memory by
 * the fused kernel (k_ow_seed_climate with one cell per seed), k_ow_search_first keeps the candidates that
 * pass; only those get their lattices written to HBM (launch_setup) and k_search_rest checks the remaining
 * observations.  Nether and End: setup for the chunk, then k_search_rest from the first observation.
 * k_search_rest stops at a candidate's first failing observation, like the reference; reached[j] counts
 * candidates that passed exactly j observations, and candidates passing all are returned sorted as
 * unsigned. */
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <mutex>
#include <vector>

#include "../../include/mcgen_gb300.h"
#include "abi_internal.h"
#include "launch.h"
#include "prof.h"
#include "search.cuh"

static_assert(sizeof(MgObs) == sizeof(McGb300Obs) && sizeof(MgObs) == 32, "observation layout");

namespace mg {
namespace {

/* candidates [off, off + n) of a source and, when `pts` is set, each one's cell of observation o */
__global__ void k_search_cells(int kind, const int64_t *__restrict__ list, uint64_t base, uint64_t off, int n, MgObs o,
                               int64_t *__restrict__ seeds, int32_t *__restrict__ pts) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int64_t seed = search_seed(kind, list, base, off + (uint64_t)i);
    seeds[i] = seed;
    if (pts) {
        int64_t hs = 0;
        bool have = false;
        int qx, qy, qz;
        obs_cell(o, seed, hs, have, qx, qy, qz);
        pts[3 * i] = qx;
        pts[3 * i + 1] = qy;
        pts[3 * i + 2] = qz;
    }
}

/* observations j0 .. nobs-1 of every seed, stopping at the first that fails; one thread per seed, its
 * lattices from `states` through L1 */
template <bool FM, int DIM>
__global__ void __launch_bounds__(128) k_search_rest(const __grid_constant__ MgWorldDesc W, const MgTreeNode *__restrict__ tree,
                                                     const MgLattice *__restrict__ states, const int64_t *__restrict__ seeds,
                                                     int ns, const MgObs *__restrict__ obs, int nobs, int j0, int ties,
                                                     int64_t *__restrict__ found, unsigned *__restrict__ nfound,
                                                     unsigned maxfound, unsigned long long *__restrict__ reached) {
    __shared__ MgSpline S;
    __shared__ unsigned hist[MG_MAX_OBS + 1];
    for (int i = threadIdx.x; i <= nobs; i += blockDim.x) hist[i] = 0;
    if (DIM == MG_OVERWORLD) {
        const uint4 *c = reinterpret_cast<const uint4 *>(&W.spline);
        uint4 *d = reinterpret_cast<uint4 *>(&S);
        for (int i = threadIdx.x; i < (int)(sizeof(MgSpline) / 16); i += blockDim.x) d[i] = c[i];
    }
    __syncthreads();
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g < ns) {
        const int64_t seed = seeds[g];
        const MgLattice *T = states + (size_t)g * W.ntables;
        int64_t hs = 0;
        bool have = false;
        int j = j0;
        for (; j < nobs; j++) {
            const MgObs &o = obs[j];
            int qx, qy, qz;
            obs_cell(o, seed, hs, have, qx, qy, qz);
            bool ok;
            if (DIM == MG_END) {
                ok = end_accept<FM>(W, T->p, o, qx, qz);
            } else {
                int32_t tg[6];
                cell_target<FM, DIM>(W, S, T, qx, qy, qz, tg);
                ok = obs_accept(o, tree, tg, ties != 0);
            }
            if (!ok) break;
        }
        atomicAdd(&hist[j], 1u);
        if (j == nobs) {
            const unsigned k = atomicAdd(nfound, 1u);
            if (k < maxfound) found[k] = seed;
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i <= nobs; i += blockDim.x)
        if (hist[i]) atomicAdd(&reached[i], (unsigned long long)hist[i]);
}

template <bool FM>
int rest_t(const MgWorldDesc &W, const MgTreeNode *tree, const MgLattice *states, const int64_t *seeds, int ns,
           const MgObs *obs, int nobs, int j0, int ties, int64_t *found, unsigned *nfound, unsigned maxfound,
           unsigned long long *reached, cudaStream_t st) {
    const unsigned grid = (unsigned)((ns + 127) / 128);
    ProfScope ps_(K_SEARCH_REST, st);
    if (W.dim == MG_OVERWORLD)
        k_search_rest<FM, MG_OVERWORLD><<<grid, 128, 0, st>>>(W, tree, states, seeds, ns, obs, nobs, j0, ties, found, nfound, maxfound, reached);
    else if (W.dim == MG_NETHER)
        k_search_rest<FM, MG_NETHER><<<grid, 128, 0, st>>>(W, tree, states, seeds, ns, obs, nobs, j0, ties, found, nfound, maxfound, reached);
    else
        k_search_rest<FM, MG_END><<<grid, 128, 0, st>>>(W, tree, states, seeds, ns, obs, nobs, j0, ties, found, nfound, maxfound, reached);
    count_launch_external();
    return (int)cudaGetLastError();
}
int launch_rest(const MgWorldDesc &W, const MgTreeNode *tree, const MgLattice *states, const int64_t *seeds, int ns,
                const MgObs *obs, int nobs, int j0, int ties, int64_t *found, unsigned *nfound, unsigned maxfound,
                unsigned long long *reached, cudaStream_t st) {
    if (ns <= 0) return 0;
    return W.fmode ? rest_t<true>(W, tree, states, seeds, ns, obs, nobs, j0, ties, found, nfound, maxfound, reached, st)
                   : rest_t<false>(W, tree, states, seeds, ns, obs, nobs, j0, ties, found, nfound, maxfound, reached, st);
}

int cuda_code(cudaError_t e) {
    return e == cudaSuccess ? MCGEN_OK : e == cudaErrorMemoryAllocation ? MCGEN_E_NOMEM : MCGEN_E_INTERNAL;
}

/* stream-ordered device scratch of the search, freed on the same stream */
struct Scratch {
    cudaStream_t st;
    std::vector<void *> ptrs;
    explicit Scratch(cudaStream_t s) : st(s) {}
    ~Scratch() {
        for (void *p : ptrs) cudaFreeAsync(p, st);
    }
    template <typename T>
    cudaError_t get(T **p, size_t count) {
        void *q = nullptr;
        cudaError_t e = cudaMallocAsync(&q, std::max<size_t>(count, 1) * sizeof(T), st);
        if (e == cudaSuccess) ptrs.push_back(q);
        *p = (T *)q;
        return e;
    }
};

}  // namespace
}  // namespace mg

extern "C" {

MCGEN_API int mcgen_gb300_search(const McWorld *w, int kind, const int64_t *list, uint64_t base, uint64_t n,
                                 const McGb300Obs *obs, int nobs, int ties, int64_t *found, uint32_t max_found,
                                 uint32_t *n_found, uint64_t *reached, double *ms) {
    if (!w || !obs || nobs < 1 || nobs > MG_MAX_OBS || !reached || !n_found || (max_found && !found)) return MCGEN_E_ARG;
    if (kind < MCGEN_SEEDS_LIST || kind > MCGEN_SEEDS_RANGE || (kind == MCGEN_SEEDS_LIST && n && !list)) return MCGEN_E_ARG;
    for (int j = 0; j < nobs; j++)
        if ((obs[j].flags & 0xFF) > 12 || (obs[j].flags & ~(MCGEN_OBS_BLOCK | 0xFF))) return MCGEN_E_ARG;
    std::lock_guard<std::mutex> lk(mg::abi_lock());
    if (!mg::abi_device_ready()) return MCGEN_E_UNSUPPORTED;
    int rc = mg::abi_world_device(const_cast<McWorld *>(w));
    if (rc) return rc;
    const MgWorldDesc &W = w->desc;
    const bool ow = W.dim == MG_OVERWORLD;
    if (ow && !mg::fused_supported(W)) return MCGEN_E_UNSUPPORTED;
    const uint64_t total = kind == MCGEN_SEEDS_STRUCTURE ? 65536u : n;
    /* candidates per chunk, and survivors per lattice batch (Overworld: 16.2 KB of lattices per seed) */
    const int CH = W.dim == MG_NETHER ? (1 << 18) : (1 << 20);
    const int SB = 1 << 16;
    cudaStream_t st = mg::abi_stream();
    mg::Scratch sc(st);
    MgObs *d_obs;
    int64_t *d_seeds, *d_surv = nullptr, *d_found, *d_list = nullptr;
    int32_t *d_pts = nullptr;
    void *d_clim = nullptr;
    MgLattice *d_states;
    unsigned *d_cnt; /* [0] survivors of the chunk, [1] found */
    unsigned long long *d_reached;
    cudaError_t e = sc.get(&d_obs, (size_t)nobs);
    if (!e) e = sc.get(&d_seeds, (size_t)CH);
    if (!e) e = sc.get(&d_found, (size_t)max_found);
    if (!e) e = sc.get(&d_cnt, 2);
    if (!e) e = sc.get(&d_reached, (size_t)nobs + 1);
    if (!e && kind == MCGEN_SEEDS_LIST) e = sc.get(&d_list, (size_t)CH);
    if (!e && ow) {
        e = sc.get(&d_pts, (size_t)CH * 3);
        if (!e) e = sc.get(&d_surv, (size_t)CH);
        if (!e) e = sc.get((uint8_t **)&d_clim, mg::fused_scratch_bytes(W, CH));
        if (!e) e = sc.get(&d_states, (size_t)SB * W.ntables);
    } else if (!e) {
        e = sc.get(&d_states, (size_t)CH * W.ntables);
    }
    if (!e) e = cudaMemcpyAsync(d_obs, obs, sizeof(MgObs) * (size_t)nobs, cudaMemcpyHostToDevice, st);
    if (!e) e = cudaMemsetAsync(d_cnt, 0, 2 * sizeof(unsigned), st);
    if (!e) e = cudaMemsetAsync(d_reached, 0, sizeof(unsigned long long) * ((size_t)nobs + 1), st);
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (!e) e = cudaEventCreate(&e0);
    if (!e) e = cudaEventCreate(&e1);
    if (!e) e = cudaEventRecord(e0, st);
    MgObs o0;
    memcpy(&o0, &obs[0], sizeof o0);
    for (uint64_t s0 = 0; !e && !rc && s0 < total; s0 += (uint64_t)CH) {
        const int m = (int)std::min<uint64_t>((uint64_t)CH, total - s0);
        const int64_t *src = nullptr;
        if (kind == MCGEN_SEEDS_LIST) {
            e = cudaMemcpyAsync(d_list, list + s0, sizeof(int64_t) * (size_t)m, cudaMemcpyHostToDevice, st);
            src = d_list;
        }
        if (e) break;
        const uint64_t off = kind == MCGEN_SEEDS_LIST ? 0 : s0;
        mg::count_launch_external();
        {
            mg::ProfScope ps_(mg::K_SEARCH_CELLS, st);
            mg::k_search_cells<<<(unsigned)((m + 127) / 128), 128, 0, st>>>(kind, src, base, off, m, o0, d_seeds, ow ? d_pts : nullptr);
        }
        if (!ow) {
            rc = mg::launch_setup(W, d_seeds, m, d_states, st);
            if (!rc) rc = mg::launch_rest(W, w->d_tree, d_states, d_seeds, m, d_obs, nobs, 0, ties, d_found, d_cnt + 1,
                                          max_found, d_reached, st);
            continue;
        }
        e = cudaMemsetAsync(d_cnt, 0, sizeof(unsigned), st);
        if (!e) rc = mg::launch_ow_search_first(W, w->d_tree, d_seeds, m, d_pts, o0, ties, d_clim, d_surv, d_cnt, d_reached, st);
        unsigned ns = 0;
        if (!e && !rc) e = cudaMemcpyAsync(&ns, d_cnt, sizeof(unsigned), cudaMemcpyDeviceToHost, st);
        if (!e && !rc) e = cudaStreamSynchronize(st);
        for (unsigned b0 = 0; !e && !rc && b0 < ns; b0 += (unsigned)SB) {
            const int mb = (int)std::min<unsigned>((unsigned)SB, ns - b0);
            if (nobs > 1) rc = mg::launch_setup(W, d_surv + b0, mb, d_states, st);
            if (!rc) rc = mg::launch_rest(W, w->d_tree, d_states, d_surv + b0, mb, d_obs, nobs, 1, ties, d_found, d_cnt + 1,
                                          max_found, d_reached, st);
        }
    }
    if (!e && !rc) e = cudaEventRecord(e1, st);
    unsigned nf = 0;
    std::vector<unsigned long long> hr((size_t)nobs + 1, 0);
    if (!e && !rc) e = cudaMemcpyAsync(&nf, d_cnt + 1, sizeof(unsigned), cudaMemcpyDeviceToHost, st);
    if (!e && !rc) e = cudaMemcpyAsync(hr.data(), d_reached, sizeof(unsigned long long) * hr.size(), cudaMemcpyDeviceToHost, st);
    if (!e && !rc) e = cudaStreamSynchronize(st);
    const unsigned nw = std::min<unsigned>(nf, max_found);
    if (!e && !rc && nw) e = cudaMemcpy(found, d_found, sizeof(int64_t) * nw, cudaMemcpyDeviceToHost);
    float t = 0.0f;
    if (!e && !rc && ms) e = cudaEventElapsedTime(&t, e0, e1);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (rc) return MCGEN_E_INTERNAL;
    if (e) return mg::cuda_code(e);
    std::sort(found, found + nw, [](int64_t a, int64_t b) { return (uint64_t)a < (uint64_t)b; });
    for (int j = 0; j <= nobs; j++) reached[j] = hr[(size_t)j];
    *n_found = nw;
    if (ms) *ms = t;
    return MCGEN_OK;
}

/* half-width of the End window that decides membership in `mask` (engine/cuda/mc_gpu.cuh:640-652): the
 * lowest class threshold at which membership changes bounds the islands that can matter */
MCGEN_API int mcgen_gb300_obs_end_radius(const McWorld *w, const uint64_t mask[2]) {
    if (!w || !mask) return -1;
    static const int order[4] = {3, 4, 2, 1}; /* small islands, barrens, midlands, highlands */
    static const int th[3] = {-20, 0, 40};
    int m[4];
    for (int i = 0; i < 4; i++) {
        const int b = w->desc.end_ids[order[i]];
        m[i] = (int)((mask[b >> 6] >> (b & 63)) & 1u);
    }
    int T = 1000;
    for (int i = 0; i < 3; i++)
        if (m[i] != m[i + 1] && th[i] < T) T = th[i];
    if (T == 1000) return 0;
    const double dmax = (101.0 - (double)T) / 9.0;
    const int rad = (int)((dmax + 1.0) / 2.0);
    return rad > 12 ? 12 : rad;
}

}  // extern "C"
