/* batch.cu -- many biome-map requests of uneven size in one persistent launch.
 *
 * A request is (world: version + dimension + preset, seed, quart region qx0..qx0+nx-1 x qz0..qz0+nz-1 at
 * quart y, tie rule).  The host splits every request into tiles -- 128 quart cells (8 x 16; the autotuner
 * picks the register budget) for Overworld and Nether, 8 x 8 chunks (32 x 32 quart cells) for the End --
 * and numbers them.  k_batch runs one CTA per SM slot for the whole batch; each CTA takes the next tile
 * from a device counter (the work queue), finds its request among the requests' first-tile numbers, stages
 * that request's seed lattices in shared memory when they differ from the previous tile's, and computes the
 * tile (for a double-branch Overworld tile, first the shift noises' per-column and per-row splits).  Uneven
 * requests therefore cost no idle SMs and no per-request launches.
 *
 * The seed lattices of every (world, seed) of the batch are built beforehand by k_setup_list_* into a
 * state pool (the served form keeps that pool across batches as a device cache).
 *
 * End tiles: the class of chunk (cx, cz) needs the island noise over the 25 x 25 chunk cells around it
 * (engine/mc_end.h:66-93).  An 8 x 8-chunk tile evaluates the (8+24)^2 simplex cells of its window once
 * into shared memory (island flag and size) instead of 64 x 625 evaluations, then each chunk scans its
 * window there.
 */
#include <cuda_runtime.h>
#include <stdint.h>

#include "batch.h"
#include "climate.cuh"
#include "endtile.cuh"
#include "launch.h"
#include "prof.h"

namespace mg {

#define BNT 128        /* threads per CTA: one quart cell per thread in Overworld / Nether tiles */

/* ---------------------------------------------------------------- setup of a list of (world, seed) */
#define LNT 128
__device__ __forceinline__ void lst_swap(uint8_t *mine, int i, int j) {
    uint8_t *a = mine + (i >> 2) * (4 * LNT) + (i & 3);
    uint8_t *b = mine + (j >> 2) * (4 * LNT) + (j & 3);
    uint8_t x = *a, y = *b;
    *a = y;
    *b = x;
}
__device__ __forceinline__ void lst_store(uint32_t (*perm)[LNT], int t, MgLattice &h, MgLattice *L, bool dbl) {
    lattice_header(h, dbl);
    const uint4 *src = reinterpret_cast<const uint4 *>(&h);
    uint4 *dst = reinterpret_cast<uint4 *>(L);
    for (int q = 0; q < MG_LAT_HDR_WORDS; q++) dst[q] = src[q];
    uint4 *dp = reinterpret_cast<uint4 *>(L->p);
    for (int q = 0; q < 16; q++) dp[q] = make_uint4(perm[4 * q][t], perm[4 * q + 1][t], perm[4 * q + 2][t], perm[4 * q + 3][t]);
}
/* Overworld entries: one thread per (entry, lattice). */
__global__ void __launch_bounds__(LNT) k_setup_list_xo(const MgWorldDesc *__restrict__ worlds, const MgSetupEntry *__restrict__ ent,
                                                       int n, const int *__restrict__ first_lattice, long long total,
                                                       MgLattice *__restrict__ pool) {
    __shared__ uint32_t perm[64][LNT];
    const int t = threadIdx.x;
    const long long g = (long long)blockIdx.x * LNT + t;
    if (g >= total) return;
    int lo = 0, hi = n - 1; /* entry e with first_lattice[e] <= g < first_lattice[e+1] */
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (first_lattice[mid] <= g) lo = mid; else hi = mid - 1;
    }
    const MgSetupEntry &E = ent[lo];
    const MgWorldDesc &W = worlds[E.world];
    const int j = (int)(g - first_lattice[lo]);
    int i = 0;
    while (i < MG_OW_NOISES - 1 && j >= W.noise[i + 1].base) i++;
    const MgNoise &N = W.noise[i];
    const int r = j - N.base, st = r >= N.nlev, k = r - st * N.nlev;
    Xo root = xo_from_seed(E.seed);
    uint64_t plo = xo_next(root), phi = xo_next(root);
    Xo nr = xo_make(W.nhl[i] ^ plo, W.nhh[i] ^ phi);
    uint64_t a = xo_next(nr), b = xo_next(nr);
    if (st) { a = xo_next(nr); b = xo_next(nr); }
    Xo x = xo_make(N.hlo[k] ^ a, N.hhi[k] ^ b);
    MgLattice h;
    h.ox = xo_double(x) * 256.0;
    h.oy = xo_double(x) * 256.0;
    h.oz = xo_double(x) * 256.0;
    for (int w = 0; w < 64; w++) perm[w][t] = 0x03020100u + 0x04040404u * (uint32_t)w;
    uint8_t *mine = reinterpret_cast<uint8_t *>(&perm[0][t]);
    for (int q = 0; q < 256; q++) lst_swap(mine, q, q + xo_int(x, 256u - (uint32_t)q));
    lst_store(perm, t, h, pool + E.slot + j, !W.fmode);
}
/* Nether entries: one thread per (entry, noise); End entries: one thread per entry. */
__device__ __forceinline__ void lst_legacy(uint64_t &s, uint32_t (*perm)[LNT], int t, MgLattice *L, bool dbl) {
    MgLattice h;
    h.ox = lcg_double(s) * 256.0;
    h.oy = lcg_double(s) * 256.0;
    h.oz = lcg_double(s) * 256.0;
    for (int w = 0; w < 64; w++) perm[w][t] = 0x03020100u + 0x04040404u * (uint32_t)w;
    uint8_t *mine = reinterpret_cast<uint8_t *>(&perm[0][t]);
    for (int q = 0; q < 256; q++) lst_swap(mine, q, q + lcg_int(s, 256 - q));
    if (L) lst_store(perm, t, h, L, dbl);
}
__global__ void __launch_bounds__(LNT) k_setup_list_legacy(const MgWorldDesc *__restrict__ worlds,
                                                           const MgSetupEntry *__restrict__ ent, int n,
                                                           MgLattice *__restrict__ pool) {
    __shared__ uint32_t perm[64][LNT];
    const int t = threadIdx.x;
    const long long g = (long long)blockIdx.x * LNT + t;
    if (g >= 2LL * n) return;
    const MgSetupEntry &E = ent[g >> 1];
    const MgWorldDesc &W = worlds[E.world];
    const int nz = (int)(g & 1);
    const MgNoise &N = W.nether[nz];
    uint64_t st = lcg_init((int64_t)((uint64_t)E.seed + (uint64_t)nz));
    MgLattice *T = pool + E.slot + N.base;
    int slot[MG_MAX_OCT];
    for (int q = 0; q < MG_MAX_OCT; q++) slot[q] = -1;
    for (int k = 0; k < N.nlev; k++) slot[N.idx[k]] = k;
    const int zero = -N.first;
    for (int stack = 0; stack < 2; stack++) {
        MgLattice *S = T + stack * N.nlev;
        const bool keep_zero = zero >= 0 && zero < N.octs && slot[zero] >= 0;
        lst_legacy(st, perm, t, keep_zero ? S + slot[zero] : nullptr, !W.fmode);
        for (int q = zero - 1; q >= 0; q--) {
            if (q < N.octs && slot[q] >= 0) lst_legacy(st, perm, t, S + slot[q], !W.fmode);
            else st = lcg_jump(st, 262);
        }
    }
}
__global__ void __launch_bounds__(LNT) k_setup_list_end(const MgSetupEntry *__restrict__ ent, int n, MgLattice *__restrict__ pool) {
    __shared__ uint32_t perm[64][LNT];
    const long long g = (long long)blockIdx.x * LNT + threadIdx.x;
    if (g >= n) return;
    uint64_t st = lcg_jump(lcg_init(ent[g].seed), 17292);
    lst_legacy(st, perm, threadIdx.x, pool + ent[g].slot, false); /* the End reads the permutation only */
}

/* ---------------------------------------------------------------- the persistent batch kernel */
/* The lattices of an Overworld/Nether request (with an Overworld tile's shift table) and the
 * End's scratch are never live in the same tile, so they share storage: 21 KB per CTA, which leaves the
 * register budget as the occupancy limit (up to 9 CTAs per SM). */
struct BatchEnd {
    uint8_t endp[256];
    EndTile tile;
};
/* the lattices of an Overworld/Nether request, and the shift table of an Overworld tile (double or float
 * branch) */
struct BatchLat {
    MgLattice lat[MG_MAX_TABLES];
    union {
        ShiftTable<8, BNT / 8> shift;   /* double-branch Overworld tile */
        ShiftTableF<8, BNT / 8> shiftf; /* float-branch Overworld tile */
    };
};
struct BatchSmem {
    union {
        BatchLat o;
        BatchEnd end;
    };
    WarpTreeScratch wt[BNT / 32]; /* each warp's R-tree candidate list (Overworld, ENGINE rule) */
    PendSink sink;  /* where double-branch Overworld cells left to the exact evaluation are recorded */
    double depth_g; /* the double-branch Overworld tile's depth gradient (depth_grad_d) */
    int tile, req, state;
};

/* a biome id to the output: written once and never read back by the kernel, so stored with the streaming
 * (evict-first) policy, which keeps the streamed output from evicting the threads' local memory from L2 */
__device__ __forceinline__ void put_id(uint8_t *p, int v) { __stcs(p, (unsigned char)v); }

/* tab, tabf: the tile's shift table (double- or float-branch Overworld, ENGINE rule) or null; g: with the
 * double branch's table, the tile's depth gradient.  Each code path's cells (and the End's tiles, batch_end) are a function of their own, out of
 * line: the persistent kernel is then a dispatcher, and each path's registers are allocated for that path
 * alone (measured 0.3 % faster on the mixed batch than all paths inlined into the kernel). */
template <bool FM, int DIM, int TILE_W>
__device__ __noinline__ void batch_cells(const MgWorldDesc &W, const MgSpline &S, const MgLattice *T,
                                            const MgTreeNode *tree, const MgBatchReq &R, int tx0, int tz0,
                                            const ShiftTable<8, BNT / 8> *tab, const ShiftTableF<8, BNT / 8> *tabf,
                                            double g, WarpTreeScratch *wt, const PendSink *sink, uint8_t *out) {
    const int col = threadIdx.x % TILE_W, row = threadIdx.x / TILE_W;
    const int ix = tx0 + col, iz = tz0 + row;
    const bool in = ix < R.nx && iz < R.nz;
    const int qx = R.qx0 + ix, qz = R.qz0 + iz;
    if (R.tie == MG_TIE_CHUNK_CELL) { /* the request's rule: the same for the whole CTA */
        if (in) put_id(out + R.out_off + (size_t)iz * R.nx + ix, cell_chunk<FM, DIM>(W, S, T, tree, qx, R.qy, qz));
        return;
    }
    int32_t tg[6] = {0, 0, 0, 0, 0, 0};
    const int64_t o = R.out_off + (int64_t)iz * R.nx + ix;
    if (!FM && DIM == MG_OVERWORLD && TILE_W == 8 && tab) {
        /* a cell whose screen left a value to the exact evaluation is recorded for the second launch (the
         * double branch's tree search is per lane, so the lane may leave here) */
        if (in && !climate_ow_d_tab_defer(W, S, T, *tab, col, row, qx, R.qy, qz, g, tg, sink, o)) return;
    } else if (FM && DIM == MG_OVERWORLD && TILE_W == 8 && tabf) {
        if (in) climate_ow_f_tab(W, S, T, *tabf, col, row, qx, R.qy, qz, tg);
    } else if (in) {
        cell_target<FM, DIM>(W, S, T, qx, R.qy, qz, tg);
    }
    int leaf;
    /* one pruned walk of the tree per warp of 8 x 4 cells for wide trees (built only into the float branch's
     * code: the double branch's versions, 26.1 and 26.2, have 6 children per node) */
    if (FM && DIM == MG_OVERWORLD && W.tree_fanout >= MG_WARP_TREE_FANOUT) {
        leaf = tree_search_warp(tree, tg, in, wt[threadIdx.x >> 5]);
    } else {
        uint64_t d;
        leaf = in ? tree_search(tree, tg, -1, d) : -1;
    }
    if (in) put_id(out + o, tree[leaf].biome);
}

/* End tile: chunks [cx0, cx0 + END_TC) x [cz0, cz0 + END_TC) counted from the chunk of the request's
 * first cell; the tile writes the request's cells that lie in those chunks. */
template <bool FM>
__device__ __noinline__ void batch_end(const MgWorldDesc &W, BatchSmem &sm, const MgBatchReq &R, int tcx, int tcz,
                                          uint8_t *out) {
    const int cx0 = (R.qx0 >> 2) + tcx * END_TC, cz0 = (R.qz0 >> 2) + tcz * END_TC;
    end_tile_classes<FM>(sm.end.endp, W.end_f2, W.end_g2, cx0, cz0, sm.end.tile);
    for (int i = threadIdx.x; i < 16 * END_TC * END_TC; i += blockDim.x) {
        const int qx = 4 * cx0 + i % (4 * END_TC), qz = 4 * cz0 + i / (4 * END_TC);
        const int ix = qx - R.qx0, iz = qz - R.qz0;
        if (ix < 0 || iz < 0 || ix >= R.nx || iz >= R.nz) continue;
        put_id(out + R.out_off + (size_t)iz * R.nx + ix,
               W.end_ids[sm.end.tile.cls[(i / (16 * END_TC)) * END_TC + (i % (4 * END_TC)) / 4]]);
    }
}

/* The request holding tile `tile`: the last r with reqs[r].tile0 <= tile (tile0 is non-decreasing and
 * reqs[0].tile0 == 0), found by the 32 lanes of a warp in rounds of 32 probes -- the probes that are <= tile
 * form a prefix, whose length narrows the range 32-fold -- so 3 rounds of loads for 10,000 requests where a
 * binary search by one thread made 14 dependent ones while the CTA waited. */
__device__ __forceinline__ int find_req(const MgBatchReq *__restrict__ reqs, int nreq, long long tile) {
    const int lane = threadIdx.x & 31;
    int lo = 0, hi = nreq - 1;
    while (hi > lo) {
        const int step = (hi - lo + 31) / 32;
        const int p = lo + (lane + 1) * step;
        const unsigned m = __ballot_sync(0xFFFFFFFFu, p <= hi && reqs[p].tile0 <= tile);
        lo += __popc(m) * step;
        hi = min(hi, lo + step - 1);
    }
    return lo;
}

/* TILE_W: tile width in cells (tiles are 128 cells); MINB: resident CTAs per SM the register allocation
 * is sized for (6: 80 registers, 7: 72, 8: 64, 9: 56) */
template <int TILE_W, int MINB>
__global__ void __launch_bounds__(BNT, MINB) k_batch(const MgWorldDesc *__restrict__ worlds, const MgTreeNode *const *__restrict__ trees,
                                               const MgBatchReq *__restrict__ reqs, int nreq, long long ntiles,
                                               const MgLattice *__restrict__ pool, unsigned long long *__restrict__ counter,
                                               MgPending *__restrict__ pend, long long pend_cap,
                                               uint8_t *__restrict__ out) {
    extern __shared__ uint4 smem_raw[];
    BatchSmem &sm = *reinterpret_cast<BatchSmem *>(smem_raw);
    if (threadIdx.x == 0) {
        sm.state = -1;
        sm.sink.rec = pend;
        sm.sink.count = counter + 1;
        sm.sink.cap = pend ? pend_cap : 0;
    }
    for (;;) {
        __syncthreads();
        if (threadIdx.x < 32) { /* warp 0 takes the next tile and finds its request */
            long long tile = 0;
            if (threadIdx.x == 0) tile = (long long)atomicAdd(counter, 1ULL);
            tile = __shfl_sync(0xFFFFFFFFu, tile, 0);
            const int r = tile < ntiles ? find_req(reqs, nreq, tile) : -1;
            if (threadIdx.x == 0) {
                sm.tile = (int)(r >= 0 ? tile - reqs[r].tile0 : -1);
                sm.req = r;
                if (r >= 0) {
                    sm.sink.world = reqs[r].world;
                    sm.sink.state = reqs[r].state;
                }
            }
        }
        __syncthreads();
        const int r = sm.req;
        if (r < 0) return;
        const MgBatchReq R = reqs[r];
        const MgWorldDesc &W = worlds[R.world];
        /* stage the request's lattices when they change (the world's offset spline, about 11 nodes read per
         * sample, is read in place through L1: kept out of shared memory, it leaves room for 9 CTAs per SM) */
        const bool new_state = R.state != sm.state;
        if (new_state) {
            if (W.dim == MG_END) {
                for (int i = threadIdx.x; i < 256; i += BNT) sm.end.endp[i] = pool[R.state].p[i];
            } else {
                const uint4 *a = reinterpret_cast<const uint4 *>(pool + R.state);
                uint4 *b = reinterpret_cast<uint4 *>(sm.o.lat);
                for (int i = threadIdx.x; i < W.ntables * (int)(sizeof(MgLattice) / 16); i += BNT) b[i] = a[i];
            }
        }
        __syncthreads();
        if (threadIdx.x == 0) sm.state = R.state;
        const int tile = sm.tile;
        if (W.dim == MG_END) {
            const int ncx = ((R.qx0 + R.nx - 1) >> 2) - (R.qx0 >> 2) + 1;
            const int tw = (ncx + END_TC - 1) / END_TC;
            if (W.fmode) batch_end<true>(W, sm, R, tile % tw, tile / tw, out);
            else batch_end<false>(W, sm, R, tile % tw, tile / tw, out);
            continue;
        }
        constexpr int TILE_H = BNT / TILE_W;
        const int tw = (R.nx + TILE_W - 1) / TILE_W;
        const int tx0 = (tile % tw) * TILE_W, tz0 = (tile / tw) * TILE_H;
        const MgTreeNode *tree = trees[R.world];
        if (W.fmode) {
            if (W.dim == MG_OVERWORLD) {
                /* the tile's shift splits, computed once per column and row (ENGINE rule) */
                const bool tab = TILE_W == 8 && R.tie != MG_TIE_CHUNK_CELL && shift_table_ok(W);
                if (tab) {
                    shift_table_fill_f<8, BNT / 8, BNT>(W.noise[0], sm.o.lat, R.qx0 + tx0, R.qz0 + tz0, sm.o.shiftf);
                    __syncthreads();
                }
                batch_cells<true, MG_OVERWORLD, TILE_W>(W, W.spline, sm.o.lat, tree, R, tx0, tz0, nullptr,
                                                        tab ? &sm.o.shiftf : nullptr, 0.0, sm.wt, &sm.sink, out);
            } else {
                batch_cells<true, MG_NETHER, TILE_W>(W, W.spline, sm.o.lat, tree, R, tx0, tz0, nullptr, nullptr, 0.0, sm.wt,
                                                     &sm.sink, out);
            }
        } else if (W.dim == MG_OVERWORLD) {
            /* the tile's shift splits, computed once per column and row (ENGINE rule) */
            const bool tab = TILE_W == 8 && R.tie != MG_TIE_CHUNK_CELL && shift_table_ok(W);
            if (tab) {
                shift_table_fill<8, BNT / 8, BNT>(W.noise[0], sm.o.lat, R.qx0 + tx0, R.qz0 + tz0, sm.o.shift);
                if (threadIdx.x == BNT - 1) sm.depth_g = depth_grad_d(W, R.qy * 4); /* a thread with fewer entries */
                __syncthreads();
            }
            batch_cells<false, MG_OVERWORLD, TILE_W>(W, W.spline, sm.o.lat, tree, R, tx0, tz0, tab ? &sm.o.shift : nullptr,
                                                     nullptr, tab ? sm.depth_g : 0.0, sm.wt, &sm.sink, out);
        } else {
            batch_cells<false, MG_NETHER, TILE_W>(W, W.spline, sm.o.lat, tree, R, tx0, tz0, nullptr, nullptr, 0.0, sm.wt,
                                                  &sm.sink, out);
        }
    }
}

/* The recorded cells (MgPending): one thread each, the exact evaluation of the values the screen left, the
 * climate finish and the R-tree search (the lanes' targets are unrelated), then the cell's output byte. */
__global__ void __launch_bounds__(128) k_batch_exact(const MgWorldDesc *__restrict__ worlds,
                                                     const MgTreeNode *const *__restrict__ trees,
                                                     const MgLattice *__restrict__ pool,
                                                     const MgPending *__restrict__ pend,
                                                     const unsigned long long *__restrict__ npend, long long cap,
                                                     uint8_t *__restrict__ out) {
    const long long n = min((long long)*npend, cap);
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const MgPending P = pend[i];
        const MgWorldDesc &W = worlds[P.world];
        int32_t tg[6];
        pending_targets(W, pool + P.state, P, tg);
        const MgTreeNode *tree = trees[P.world];
        uint64_t d;
        put_id(out + P.out, tree[tree_search_scattered(tree, tg, -1, d)].biome);
    }
}

/* ---------------------------------------------------------------- host side */
long long batch_pending_cap(long long cells) { return cells > 0 ? cells / 256 + 1024 : 0; }

/* tile shapes the autotuner chooses from: tile width, and the register budget (resident CTAs per SM: 9, 7,
 * 6, 8) in k_batch's second template argument */
const int kBatchTileWidths[BATCH_SHAPES] = {8, 8, 8, 8};
static int g_resident[BATCH_SHAPES] = {0, 0, 0, 0}; /* CTAs per SM x SMs, per shape (batch_prepare) */

long long batch_tiles(int dim, int qx0, int qz0, int nx, int nz, int shape) {
    if (dim == MG_END) {
        const long long ncx = ((qx0 + nx - 1) >> 2) - (qx0 >> 2) + 1, ncz = ((qz0 + nz - 1) >> 2) - (qz0 >> 2) + 1;
        return ((ncx + END_TC - 1) / END_TC) * ((ncz + END_TC - 1) / END_TC);
    }
    const int tw = kBatchTileWidths[shape], th = BNT / tw;
    return (long long)((nx + tw - 1) / tw) * ((nz + th - 1) / th);
}

int launch_setup_list(const MgWorldDesc *d_worlds, int dim, const MgSetupEntry *d_ent, int n, const int *d_first,
                      long long total_lattices, MgLattice *d_pool, cudaStream_t st) {
    if (n <= 0) return 0;
    if (dim == MG_OVERWORLD) {
        ProfScope ps_(K_SETUP_XO, st);
        k_setup_list_xo<<<(unsigned)((total_lattices + LNT - 1) / LNT), LNT, 0, st>>>(d_worlds, d_ent, n, d_first, total_lattices, d_pool);
    } else if (dim == MG_NETHER) {
        ProfScope ps_(K_SETUP_LEGACY, st);
        k_setup_list_legacy<<<(unsigned)((2LL * n + LNT - 1) / LNT), LNT, 0, st>>>(d_worlds, d_ent, n, d_pool);
    } else {
        ProfScope ps_(K_SETUP_END, st);
        k_setup_list_end<<<(unsigned)((n + LNT - 1) / LNT), LNT, 0, st>>>(d_ent, n, d_pool);
    }
    count_launch_external();
    return (int)cudaGetLastError();
}

template <int TW, int MB>
static int prepare_t(int shape, int sms) {
    int rc = (int)cudaFuncSetAttribute(k_batch<TW, MB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(BatchSmem));
    int n = 0;
    if (!rc) rc = (int)cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_batch<TW, MB>, BNT, sizeof(BatchSmem));
    g_resident[shape] = (n > 0 ? n : 1) * sms;
    return rc;
}
/* kernel attributes (before any capture) and resident CTAs per SM of shape 0 */
int batch_prepare(int *ctas_per_sm) {
    static int prepared_dev = -1; /* the attributes are per device and set once (callers hold the ABI lock) */
    int dev = 0, sms = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (prepared_dev == dev) {
        if (ctas_per_sm) *ctas_per_sm = g_resident[0] / (sms > 0 ? sms : 1);
        return 0;
    }
    int rc = prepare_t<8, 9>(0, sms);
    if (!rc) rc = prepare_t<8, 7>(1, sms);
    if (!rc) rc = prepare_t<8, 6>(2, sms);
    if (!rc) rc = prepare_t<8, 8>(3, sms);
    if (!rc) prepared_dev = dev;
    if (ctas_per_sm) *ctas_per_sm = g_resident[0] / (sms > 0 ? sms : 1);
    return rc;
}

/* ctas: upper bound on the persistent grid (0: every resident CTA of the shape) */
int launch_batch(const MgWorldDesc *d_worlds, const MgTreeNode *const *d_trees, const MgBatchReq *d_reqs, int nreq,
                 long long ntiles, const MgLattice *d_pool, unsigned long long *d_counter, MgPending *d_pend,
                 long long pend_cap, uint8_t *d_out, int ctas, int shape, cudaStream_t st) {
    if (ntiles <= 0) return 0;
    if (shape < 0 || shape >= BATCH_SHAPES || g_resident[shape] <= 0) return (int)cudaErrorInvalidValue;
    if (!d_pend) pend_cap = 0;
    cudaError_t e = cudaMemsetAsync(d_counter, 0, 2 * sizeof(unsigned long long), st);
    if (e) return (int)e;
    int grid = g_resident[shape];
    if (ctas > 0 && ctas < grid) grid = ctas;
    if ((long long)grid > ntiles) grid = (int)ntiles;
    const size_t sm = sizeof(BatchSmem);
    {
        ProfScope ps_(K_BATCH, st);
        switch (shape) {
        case 1: k_batch<8, 7><<<grid, BNT, sm, st>>>(d_worlds, d_trees, d_reqs, nreq, ntiles, d_pool, d_counter, d_pend, pend_cap, d_out); break;
        case 2: k_batch<8, 6><<<grid, BNT, sm, st>>>(d_worlds, d_trees, d_reqs, nreq, ntiles, d_pool, d_counter, d_pend, pend_cap, d_out); break;
        case 3: k_batch<8, 8><<<grid, BNT, sm, st>>>(d_worlds, d_trees, d_reqs, nreq, ntiles, d_pool, d_counter, d_pend, pend_cap, d_out); break;
        default: k_batch<8, 9><<<grid, BNT, sm, st>>>(d_worlds, d_trees, d_reqs, nreq, ntiles, d_pool, d_counter, d_pend, pend_cap, d_out); break;
        }
    }
    count_launch_external();
    if ((e = cudaGetLastError())) return (int)e;
    if (pend_cap > 0) { /* the recorded cells; the grid covers the usual count, larger counts loop */
        ProfScope ps_(K_BATCH_EXACT, st);
        k_batch_exact<<<2 * 152, 128, 0, st>>>(d_worlds, d_trees, d_pool, d_pend, d_counter + 1, pend_cap, d_out);
        count_launch_external();
    }
    return (int)cudaGetLastError();
}

}  // namespace mg
