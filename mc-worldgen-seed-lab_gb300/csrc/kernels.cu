/* kernels.cu -- sm_103a kernels of the biome path and their host launchers.
 *
 *  per-seed setup   k_setup_xo      one thread per (seed, lattice): Xoroshiro positional seeding and the
 *                                   256-step Fisher-Yates shuffle in a bank-conflict-free shared layout
 *                   k_setup_legacy  Nether biome noises: java.util.Random, octaves from the zero octave down
 *                   k_setup_end     End island simplex: LCG(seed) jumped 17292 steps, one shuffle
 *  per-point        k_points        seeds x quart points (ENGINE tie rule), lattices read through L1
 *                   k_grid          one seed's quart grid, lattices staged in shared memory;
 *                                   ENGINE biomes or GRID_CHAIN records (leaf, fitness, tie flag, target)
 *                   k_chain_resolve GRID_CHAIN replay for the (rare) tied cells
 *                   k_blockgrid     libmcgen mcgen_biome_grid: BiomeManager zoom + chunk-cell tie chain
 *                   k_end_chunks    End island class per chunk, 8 x 8-chunk tiles (endtile.cuh)
 */
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include "climate.cuh"
#include "endtile.cuh"
#include "device.cuh"
#include "launch.h"
#include "prof.h"

using namespace mgd;

/* the cooperative 16-byte copies below rely on these layouts */
static_assert(sizeof(MgLattice) % 16 == 0, "lattice size");
static_assert(sizeof(MgSpline) % 16 == 0, "spline size");
static_assert(offsetof(MgWorldDesc, spline) % 16 == 0, "spline alignment in the description");
static_assert(sizeof(MgWorldDesc) <= 24576, "world description must fit the kernel parameter space");

namespace mg {

static long long g_launches = 0;
long long launch_count() { return g_launches; }
static inline void count_launch() { __atomic_add_fetch(&g_launches, 1, __ATOMIC_RELAXED); }
void count_launch_external() { count_launch(); }

/* ============================================================================ per-seed setup */
#define SETUP_NT 128
/* Shuffle state of thread t: byte i lives in byte (i & 3) of word perm[i >> 2][t], so every access of a
 * thread hits bank t % 32 whatever i is: the 32 lanes of a warp never conflict. */
__device__ __forceinline__ void perm_identity(uint32_t (*perm)[SETUP_NT], int t) {
    for (int w = 0; w < 64; w++) perm[w][t] = 0x03020100u + 0x04040404u * (uint32_t)w;
}
__device__ __forceinline__ void perm_swap(uint8_t *base, int t, int i, int j) {
    uint8_t *a = base + (((i >> 2) * SETUP_NT + t) << 2) + (i & 3);
    uint8_t *b = base + (((j >> 2) * SETUP_NT + t) << 2) + (j & 3);
    uint8_t x = *a, y = *b;
    *a = y;
    *b = x;
}
__device__ __forceinline__ void perm_store(uint32_t (*perm)[SETUP_NT], int t, MgLattice *L) {
    uint4 *dst = reinterpret_cast<uint4 *>(L->p);
#pragma unroll 4
    for (int q = 0; q < 16; q++) dst[q] = make_uint4(perm[4 * q][t], perm[4 * q + 1][t], perm[4 * q + 2][t], perm[4 * q + 3][t]);
}
__device__ __forceinline__ void header_store(MgLattice &h, MgLattice *L, bool dbl) {
    lattice_header(h, dbl);
    const uint4 *src = reinterpret_cast<const uint4 *>(&h);
    uint4 *dst = reinterpret_cast<uint4 *>(L);
#pragma unroll
    for (int q = 0; q < MG_LAT_HDR_WORDS; q++) dst[q] = src[q];
}

/* Overworld: lattice j of seed s; table layout noise-major, then stack, then level
 * (engine/mc_climate.h:95-106, engine/mc_noise.h:255-265). */
__global__ void __launch_bounds__(SETUP_NT) k_setup_xo(const __grid_constant__ MgWorldDesc W, const int64_t *__restrict__ seeds,
                                                       int ns, MgLattice *__restrict__ out) {
    __shared__ uint32_t perm[64][SETUP_NT];
    const int t = threadIdx.x;
    const int nt = W.ntables;
    const long long g = (long long)blockIdx.x * SETUP_NT + t;
    if (g >= (long long)ns * nt) return;
    const int s = (int)(g / nt), j = (int)(g % nt);
    int i = 0;
    while (i < MG_OW_NOISES - 1 && j >= W.noise[i + 1].base) i++;
    const MgNoise &N = W.noise[i];
    const int r = j - N.base, st = r >= N.nlev, k = r - st * N.nlev;
    Xo root = xo_from_seed(seeds[s]);
    uint64_t plo = xo_next(root), phi = xo_next(root);   /* forkPositional */
    Xo nr = xo_make(W.nhl[i] ^ plo, W.nhh[i] ^ phi);      /* fromHashOf("minecraft:<noise>") */
    uint64_t a = xo_next(nr), b = xo_next(nr);            /* first stack's forkPositional */
    if (st) { a = xo_next(nr); b = xo_next(nr); }         /* second stack's */
    Xo x = xo_make(N.hlo[k] ^ a, N.hhi[k] ^ b);           /* fromHashOf("octave_<n>") */
    MgLattice h;
    h.ox = xo_double(x) * 256.0;
    h.oy = xo_double(x) * 256.0;
    h.oz = xo_double(x) * 256.0;
    perm_identity(perm, t);
    uint8_t *base = reinterpret_cast<uint8_t *>(&perm[0][0]);
    for (int q = 0; q < 256; q++) perm_swap(base, t, q, q + xo_int(x, 256u - (uint32_t)q));
    MgLattice *L = out + g;
    header_store(h, L, !W.fmode);
    perm_store(perm, t, L);
}

/* one legacy lattice from the LCG into the thread's shuffle slot, then to `L` (if non-null) */
__device__ __forceinline__ void legacy_lattice(uint64_t &s, uint32_t (*perm)[SETUP_NT], int t, MgLattice *L, bool dbl) {
    MgLattice h;
    h.ox = lcg_double(s) * 256.0;
    h.oy = lcg_double(s) * 256.0;
    h.oz = lcg_double(s) * 256.0;
    perm_identity(perm, t);
    uint8_t *base = reinterpret_cast<uint8_t *>(&perm[0][0]);
    for (int q = 0; q < 256; q++) perm_swap(base, t, q, q + lcg_int(s, 256 - q));
    if (L) {
        header_store(h, L, dbl);
        perm_store(perm, t, L);
    }
}
/* Nether biome noises: temperature from LCG(seed), vegetation from LCG(seed + 1); each stack builds the
 * zero octave first, then octaves zero-1 .. 0, skipping 262 draws for an absent one
 * (engine/mc_noise.h:266-282, engine/cuda/mcg_host.c:49-51). */
__global__ void __launch_bounds__(SETUP_NT) k_setup_legacy(const __grid_constant__ MgWorldDesc W, const int64_t *__restrict__ seeds,
                                                           int ns, MgLattice *__restrict__ out) {
    __shared__ uint32_t perm[64][SETUP_NT];
    const int t = threadIdx.x;
    const long long g = (long long)blockIdx.x * SETUP_NT + t;
    if (g >= 2LL * ns) return;
    const int s = (int)(g >> 1), n = (int)(g & 1);
    const MgNoise &N = W.nether[n];
    uint64_t st = lcg_init((int64_t)((uint64_t)seeds[s] + (uint64_t)n));
    MgLattice *T = out + (size_t)s * W.ntables + N.base;
    int slot[MG_MAX_OCT];
    for (int q = 0; q < MG_MAX_OCT; q++) slot[q] = -1;
    for (int k = 0; k < N.nlev; k++) slot[N.idx[k]] = k;
    const int zero = -N.first;
    for (int stack = 0; stack < 2; stack++) {
        MgLattice *S = T + stack * N.nlev;
        bool keep_zero = zero >= 0 && zero < N.octs && slot[zero] >= 0;
        legacy_lattice(st, perm, t, keep_zero ? S + slot[zero] : nullptr, !W.fmode);
        for (int q = zero - 1; q >= 0; q--) {
            if (q < N.octs && slot[q] >= 0) legacy_lattice(st, perm, t, S + slot[q], !W.fmode);
            else st = lcg_jump(st, 262);
        }
    }
}
/* End: LegacyRandomSource(seed).consumeCount(17292), then the simplex lattice (engine/mc_end.h:18-22) */
__global__ void __launch_bounds__(SETUP_NT) k_setup_end(const int64_t *__restrict__ seeds, int ns, MgLattice *__restrict__ out) {
    __shared__ uint32_t perm[64][SETUP_NT];
    const int t = threadIdx.x;
    const long long g = (long long)blockIdx.x * SETUP_NT + t;
    if (g >= ns) return;
    uint64_t st = lcg_jump(lcg_init(seeds[g]), 17292);
    legacy_lattice(st, perm, t, out + g, false); /* the End reads the permutation only */
}

/* ============================================================================ sampling kernels */
/* Stage the seed-independent spline and one seed's lattices in shared memory. */
__device__ __forceinline__ void stage(const MgWorldDesc &W, const MgLattice *__restrict__ src, int n, MgLattice *dstT,
                                      MgSpline *dstS, bool spline) {
    const uint4 *a = reinterpret_cast<const uint4 *>(src);
    uint4 *b = reinterpret_cast<uint4 *>(dstT);
    for (int i = threadIdx.x; i < n * (int)(sizeof(MgLattice) / 16); i += blockDim.x) b[i] = a[i];
    if (spline) {
        const uint4 *c = reinterpret_cast<const uint4 *>(&W.spline);
        uint4 *d = reinterpret_cast<uint4 *>(dstS);
        for (int i = threadIdx.x; i < (int)(sizeof(MgSpline) / 16); i += blockDim.x) d[i] = c[i];
    }
}

/* seeds x points, ENGINE rule.  One thread per sample; lattices of the sample's seed through L1. */
template <bool FM, int DIM>
__global__ void __launch_bounds__(128) k_points(const __grid_constant__ MgWorldDesc W, const MgTreeNode *__restrict__ tree,
                                                const MgLattice *__restrict__ states, int ns,
                                                const int32_t *__restrict__ pts, int np, uint8_t *__restrict__ out,
                                                int32_t *__restrict__ targets) {
    __shared__ MgSpline S;
    if (DIM == MG_OVERWORLD) {
        const uint4 *c = reinterpret_cast<const uint4 *>(&W.spline);
        uint4 *d = reinterpret_cast<uint4 *>(&S);
        for (int i = threadIdx.x; i < (int)(sizeof(MgSpline) / 16); i += blockDim.x) d[i] = c[i];
        __syncthreads();
    }
    const long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= (long long)ns * np) return;
    const int s = (int)(g / np), p = (int)(g % np);
    const int qx = pts[3 * p], qy = pts[3 * p + 1], qz = pts[3 * p + 2];
    const MgLattice *T = states + (size_t)s * W.ntables;
    int32_t tg[6];
    if (DIM == MG_END) {
        out[g] = (uint8_t)W.end_ids[end_chunk_class(T->p, FM, (qx * 4) >> 4, (qz * 4) >> 4, W.end_f2, W.end_g2)];
        if (targets)
            for (int k = 0; k < 6; k++) targets[g * 6 + k] = 0;
        return;
    }
    cell_target<FM, DIM>(W, S, T, qx, qy, qz, tg);
    uint64_t d;
    int leaf = tree_search_scattered(tree, tg, -1, d);
    out[g] = tree[leaf].biome;
    if (targets)
        for (int k = 0; k < 6; k++) targets[g * 6 + k] = tg[k];
}

/* One seed's quart grid.  ENGINE: biome ids.  GRID_CHAIN: first minimum leaf, its fitness, tie flag and
 * the target of every cell, for k_chain_resolve. */
struct ChainRec { int32_t tg[6]; uint64_t d; int32_t leaf; int32_t tie; };
template <bool FM, int DIM, bool CHAIN>
__global__ void __launch_bounds__(128) k_grid(const __grid_constant__ MgWorldDesc W, const MgTreeNode *__restrict__ tree,
                                              const MgLattice *__restrict__ state, int qx0, int qz0, int nx, int nz,
                                              int qy, uint8_t *__restrict__ out, ChainRec *__restrict__ rec) {
    extern __shared__ uint4 smem_raw[];
    MgSpline *S = reinterpret_cast<MgSpline *>(smem_raw);
    MgLattice *T = reinterpret_cast<MgLattice *>(S + 1);
    stage(W, state, W.ntables, T, S, DIM == MG_OVERWORLD);
    /* 8 x 16-cell tiles: an Overworld tile computes its shift noises' splits once per column and row
     * (shift_table_fill, shift_table_fill_f) */
    const int tw = (nx + 7) / 8;
    const int col = threadIdx.x % 8, row = threadIdx.x / 8;
    const int tx0 = (int)(blockIdx.x % (unsigned)tw) * 8, tz0 = (int)(blockIdx.x / (unsigned)tw) * 16;
    ShiftTable<8, 16> *tab = nullptr;
    ShiftTableF<8, 16> *tabf = nullptr;
    __shared__ double depth_g; /* with a table: the depth gradient at qy (depth_grad_d), once per CTA */
    if (DIM == MG_OVERWORLD && shift_table_ok(W)) {
        __syncthreads(); /* the lattices are staged */
        if (FM) {
            tabf = reinterpret_cast<ShiftTableF<8, 16> *>(T + W.ntables);
            shift_table_fill_f<8, 16, 128>(W.noise[0], T, qx0 + tx0, qz0 + tz0, *tabf);
        } else {
            tab = reinterpret_cast<ShiftTable<8, 16> *>(T + W.ntables);
            shift_table_fill<8, 16, 128>(W.noise[0], T, qx0 + tx0, qz0 + tz0, *tab);
            if (threadIdx.x == 127) depth_g = depth_grad_d(W, qy * 4);
        }
    }
    __syncthreads();
    const int ix = tx0 + col, iz = tz0 + row;
    const bool in = ix < nx && iz < nz;
    const long long g = (long long)iz * nx + ix;
    if (FM && !CHAIN && DIM == MG_OVERWORLD && W.tree_fanout >= MG_WARP_TREE_FANOUT) { /* one pruned walk per warp */
        __shared__ WarpTreeScratch wt[4];
        int32_t tg[6] = {0, 0, 0, 0, 0, 0};
        if (in) {
            if (FM && tabf) climate_ow_f_tab(W, *S, T, *tabf, col, row, qx0 + ix, qy, qz0 + iz, tg);
            else cell_target<FM, DIM>(W, *S, T, qx0 + ix, qy, qz0 + iz, tg);
        }
        const int leaf = tree_search_warp(tree, tg, in, wt[threadIdx.x >> 5]);
        if (in) out[g] = tree[leaf].biome;
        return;
    }
    if (!in) return;
    int32_t tg[6];
    if (!FM && DIM == MG_OVERWORLD && tab) climate_ow_d_tab(W, *S, T, *tab, col, row, qx0 + ix, qy, qz0 + iz, depth_g, tg);
    else if (FM && DIM == MG_OVERWORLD && tabf) climate_ow_f_tab(W, *S, T, *tabf, col, row, qx0 + ix, qy, qz0 + iz, tg);
    else cell_target<FM, DIM>(W, *S, T, qx0 + ix, qy, qz0 + iz, tg);
    uint64_t d;
    if (CHAIN) {
        bool tied;
        const int leaf = tree_search_tie(tree, tg, d, tied);
        out[g] = tree[leaf].biome;
        ChainRec r;
        for (int k = 0; k < 6; k++) r.tg[k] = tg[k];
        r.d = d;
        r.leaf = leaf;
        r.tie = tied;
        rec[g] = r;
    } else {
        out[g] = tree[tree_search(tree, tg, -1, d)].biome;
    }
}
/* GRID_CHAIN: a tied cell takes the previous cell's leaf when that leaf is also at minimum fitness.
 * Walk back to the nearest untied cell (whose leaf is its own first minimum) and replay forward. */
__global__ void k_chain_resolve(const MgTreeNode *__restrict__ tree, const ChainRec *__restrict__ rec, long long n,
                                uint8_t *__restrict__ out) {
    const long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= n || !rec[g].tie) return;
    long long j = g - 1;
    while (j >= 0 && rec[j].tie) j--;
    int leaf = j >= 0 ? rec[j].leaf : -1;
    for (long long k = j + 1; k <= g; k++) {
        const ChainRec &r = rec[k];
        if (leaf < 0 || node_dist(tree[leaf], r.tg) != r.d) leaf = r.leaf;
    }
    out[g] = tree[leaf].biome;
}

/* CHUNK_ORDER: the chain runs chunk by chunk (chunk rows tz outer, tx inner) and, inside a chunk, over its
 * cells in the grid (z outer, x inner), across chunks: the order of the 26.3 chunk-batched climate
 * (oracle/src/v263/oracle/compat/Compat.java:168-221 in the reference).  order[pos] = cell index. */
__global__ void k_chain_order(int qx0, int qz0, int nx, int nz, int32_t *__restrict__ order) {
    const long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= (long long)nx * nz) return;
    const int qx = qx0 + (int)(g % nx), qz = qz0 + (int)(g / nx);
    const int tx = qx >> 2, tz = qz >> 2;
    const int za = max(tz * 4, qz0), zb = min(tz * 4 + 3, qz0 + nz - 1);
    const int xa = max(tx * 4, qx0), xb = min(tx * 4 + 3, qx0 + nx - 1);
    const long long pos = (long long)(za - qz0) * nx + (long long)(xa - qx0) * (zb - za + 1) +
                          (long long)(qz - za) * (xb - xa + 1) + (qx - xa);
    order[pos] = (int32_t)g;
}
/* the chain replay of k_chain_resolve along order[] */
__global__ void k_chain_resolve_ordered(const MgTreeNode *__restrict__ tree, const ChainRec *__restrict__ rec, long long n,
                                        const int32_t *__restrict__ order, uint8_t *__restrict__ out) {
    const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n || !rec[order[p]].tie) return;
    long long j = p - 1;
    while (j >= 0 && rec[order[j]].tie) j--;
    int leaf = j >= 0 ? rec[order[j]].leaf : -1;
    for (long long k = j + 1; k <= p; k++) {
        const ChainRec &r = rec[order[k]];
        if (leaf < 0 || node_dist(tree[leaf], r.tg) != r.d) leaf = r.leaf;
    }
    out[order[p]] = tree[leaf].biome;
}

/* mcgen_biome_grid: out[iz*nx+ix] = biome_at(x0 + ix*step, y, z0 + iz*step) (libmcgen/src/region.c:86-108) */
template <bool FM, int DIM>
__global__ void __launch_bounds__(128, 6) k_blockgrid(const __grid_constant__ MgWorldDesc W, const MgTreeNode *__restrict__ tree,
                                                   const MgLattice *__restrict__ state, int64_t zseed, int x0, int z0,
                                                   int nx, int nz, int step, int y, const int32_t *__restrict__ xyz,
                                                   uint8_t *__restrict__ out, const uint8_t *__restrict__ end_cls,
                                                   int ecx0, int ecz0, int encx) {
    extern __shared__ uint4 smem_raw[];
    MgSpline *S = reinterpret_cast<MgSpline *>(smem_raw);
    MgLattice *T = reinterpret_cast<MgLattice *>(S + 1);
    if (DIM != MG_END) {
        stage(W, state, W.ntables, T, S, DIM == MG_OVERWORLD);
        __syncthreads();
    }
    /* grids of a wide tree (the launcher sizes the grid in tiles for this form): the CTA takes a 16 x 8-cell tile
     * and each warp an 8 x 4 block of it, neighbours whose targets are close, so the cells' own R-tree searches share one pruned walk (the
     * chunk-cell chain, rare, stays per lane); not for scattered points or sparse grids, whose warps' targets
     * are unrelated */
    if (FM && DIM == MG_OVERWORLD && !xyz && step <= 16 && W.tree_fanout >= MG_WARP_TREE_FANOUT) {
        __shared__ WarpTreeScratch wt[4];
        const int tw = (nx + 15) / 16, w = threadIdx.x >> 5, l = threadIdx.x & 31;
        const int ix = (int)(blockIdx.x % tw) * 16 + (w & 1) * 8 + (l & 7);
        const int iz = (int)(blockIdx.x / tw) * 8 + (w >> 1) * 4 + (l >> 3);
        const bool in = ix < nx && iz < nz;
        int cx = 0, cy = 0, cz = 0;
        if (in) zoom_cell(zseed, x0 + ix * step, y, z0 + iz * step, cx, cy, cz);
        const int b = cell_chunk_warp<FM, DIM>(W, *S, T, tree, cx, cy, cz, in, wt[w]);
        if (in) out[(long long)iz * nx + ix] = (uint8_t)b;
        return;
    }
    const long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const bool in = g < (long long)nx * nz;
    if (!in) return;
    int bxk, byk, bzk;
    if (xyz) { bxk = xyz[3 * g]; byk = xyz[3 * g + 1]; bzk = xyz[3 * g + 2]; }
    else { bxk = x0 + (int)(g % nx) * step; byk = y; bzk = z0 + (int)(g / nx) * step; }
    int cx, cy, cz;
    zoom_cell(zseed, bxk, byk, bzk, cx, cy, cz);
    if (DIM == MG_END) {
        int chx = (cx * 4) >> 4, chz = (cz * 4) >> 4;
        int c = end_cls ? end_cls[(size_t)(chz - ecz0) * encx + (chx - ecx0)]
                        : end_chunk_class(state->p, FM, chx, chz, W.end_f2, W.end_g2);
        out[g] = (uint8_t)W.end_ids[c];
        return;
    }
    out[g] = (uint8_t)cell_chunk<FM, DIM>(W, *S, T, tree, cx, cy, cz);
}
/* End class of chunks [cx0, cx0+ncx) x [cz0, cz0+ncz) */
template <bool FM>
__global__ void __launch_bounds__(128) k_end_chunks(const MgLattice *__restrict__ state, int cx0, int cz0, int ncx,
                                                    int ncz, uint8_t *__restrict__ cls, double F2, double G2) {
    /* one 8 x 8-chunk tile per block (endtile.cuh) */
    __shared__ uint8_t p[256];
    __shared__ EndTile tile;
    for (int i = threadIdx.x; i < 256; i += blockDim.x) p[i] = state->p[i];
    __syncthreads();
    const int tw = (ncx + END_TC - 1) / END_TC;
    const int tx0 = cx0 + (int)(blockIdx.x % tw) * END_TC, tz0 = cz0 + (int)(blockIdx.x / tw) * END_TC;
    end_tile_classes<FM>(p, F2, G2, tx0, tz0, tile);
    if (threadIdx.x < END_TC * END_TC) {
        const int cx = tx0 + threadIdx.x % END_TC, cz = tz0 + threadIdx.x / END_TC;
        if (cx < cx0 + ncx && cz < cz0 + ncz) cls[(size_t)(cz - cz0) * ncx + (cx - cx0)] = tile.cls[threadIdx.x];
    }
}

/* ============================================================================ host launchers */
static inline unsigned blocks_for(long long n, int nt) { return (unsigned)((n + nt - 1) / nt); }
static unsigned end_tiles(int ncx, int ncz) {
    return (unsigned)(((long long)(ncx + END_TC - 1) / END_TC) * ((ncz + END_TC - 1) / END_TC));
}
static size_t grid_smem(const MgWorldDesc &W) { return sizeof(MgSpline) + (size_t)W.ntables * sizeof(MgLattice); }
/* k_grid's: the Overworld adds its tiles' shift table */
static size_t grid_smem_k(const MgWorldDesc &W) {
    return grid_smem(W) + (W.dim == MG_OVERWORLD ? (W.fmode ? sizeof(ShiftTableF<8, 16>) : sizeof(ShiftTable<8, 16>)) : 0);
}

int launch_setup(const MgWorldDesc &W, const int64_t *d_seeds, int ns, MgLattice *d_states, cudaStream_t st) {
    if (ns <= 0) return 0;
    if (W.dim == MG_OVERWORLD) {
        long long n = (long long)ns * W.ntables;
        { ProfScope ps_(K_SETUP_XO, st); k_setup_xo<<<blocks_for(n, SETUP_NT), SETUP_NT, 0, st>>>(W, d_seeds, ns, d_states); }
    } else if (W.dim == MG_NETHER) {
        { ProfScope ps_(K_SETUP_LEGACY, st); k_setup_legacy<<<blocks_for(2LL * ns, SETUP_NT), SETUP_NT, 0, st>>>(W, d_seeds, ns, d_states); }
    } else {
        { ProfScope ps_(K_SETUP_END, st); k_setup_end<<<blocks_for(ns, SETUP_NT), SETUP_NT, 0, st>>>(d_seeds, ns, d_states); }
    }
    count_launch();
    return (int)cudaGetLastError();
}

/* Overworld density functions at block points (x, y, z): out[5 i + k] = continents, erosion, ridges, offset,
 * depth as the climate sampler computes them before it rounds them to floats (engine/mc_climate.h:113-164 at
 * block coordinates; the reference Java oracle's "df" values, oracle/gen_vectors.py:76-84).  Double branch:
 * every noise by the exact double evaluation (no screen: the doubles themselves are the result); float
 * branch: the floats, widened.  One thread per point, one seed's lattices through L1. */
template <bool FM>
__global__ void __launch_bounds__(128) k_density(const __grid_constant__ MgWorldDesc W, const MgLattice *__restrict__ T,
                                                 int n, const int32_t *__restrict__ xyz, double *__restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int bx = xyz[3 * i], by = xyz[3 * i + 1], bz = xyz[3 * i + 2];
    const double X = bx * 0.25, Z = bz * 0.25, Xc = X * MG_SECOND_STACK, Zc = Z * MG_SECOND_STACK;
    double v[5];
    if (FM) {
        const float sx = nn_f_y0(W.noise[0], T, X, Z, Xc, Zc) * 4.0f; /* ShiftA (x, 0, z) */
        const float sz = nn_f_z0(W.noise[0], T, Z, X, Zc, Xc) * 4.0f; /* ShiftB (z, x, 0) */
        const double x = X + (double)sx, z = Z + (double)sz, xc = x * MG_SECOND_STACK, zc = z * MG_SECOND_STACK;
        const float c = nn_f_y0(W.noise[3], T, x, z, xc, zc);
        const float e = nn_f_y0(W.noise[4], T, x, z, xc, zc);
        const float r = nn_f_y0(W.noise[5], T, x, z, xc, zc);
        const float a = fabsf(r) + W.rf_f[0];
        const float co[4] = {c, e, r, (fabsf(a) + W.rf_f[1]) * W.rf_f[2]};
        const float off = W.off_f + spline_eval(W.spline, co);
        const int lo = min(W.grad_from_y, W.grad_to_y), hi = max(W.grad_from_y, W.grad_to_y);
        const int yy = by < lo ? lo : (by > hi ? hi : by);
        const float depth = (W.grad_from_f + (float)(yy - W.grad_from_y) * W.grad_fac_f) + off;
        v[0] = c; v[1] = e; v[2] = r; v[3] = off; v[4] = depth;
    } else {
        const double x = X + nn_d_y0(W.noise[0], T, X, Z, Xc, Zc) * 4.0;
        const double z = Z + nn_d_z0(W.noise[0], T, Z, X, Zc, Xc) * 4.0;
        const double xc = x * MG_SECOND_STACK, zc = z * MG_SECOND_STACK;
        const double c = nn_d_y0(W.noise[3], T, x, z, xc, zc);
        const double e = nn_d_y0(W.noise[4], T, x, z, xc, zc);
        const double r = nn_d_y0(W.noise[5], T, x, z, xc, zc);
        const float co[4] = {(float)c, (float)e, (float)r, (float)ridges_folded_d(W, r)};
        const double off = 0.0 + (W.off_d + (double)spline_eval(W.spline, co)) * 1.0;
        v[0] = c; v[1] = e; v[2] = r; v[3] = off; v[4] = depth_grad_d(W, by) + off;
    }
    for (int k = 0; k < 5; k++) out[5 * (size_t)i + k] = v[k];
}

template <bool FM, int DIM>
static void points_t(const MgWorldDesc &W, const MgTreeNode *tree, const MgLattice *states, int ns, const int32_t *pts,
                     int np, uint8_t *out, int32_t *tg, cudaStream_t st) {
    long long n = (long long)ns * np;
    { ProfScope ps_(K_POINTS, st); k_points<FM, DIM><<<blocks_for(n, 128), 128, 0, st>>>(W, tree, states, ns, pts, np, out, tg); }
}
int launch_points(const MgWorldDesc &W, const MgTreeNode *tree, const MgLattice *states, int ns, const int32_t *pts,
                  int np, uint8_t *out, int32_t *tg, cudaStream_t st) {
    if ((long long)ns * np <= 0) return 0;
    if (W.fmode) {
        if (W.dim == MG_OVERWORLD) points_t<true, MG_OVERWORLD>(W, tree, states, ns, pts, np, out, tg, st);
        else if (W.dim == MG_NETHER) points_t<true, MG_NETHER>(W, tree, states, ns, pts, np, out, tg, st);
        else points_t<true, MG_END>(W, tree, states, ns, pts, np, out, tg, st);
    } else {
        if (W.dim == MG_OVERWORLD) points_t<false, MG_OVERWORLD>(W, tree, states, ns, pts, np, out, tg, st);
        else if (W.dim == MG_NETHER) points_t<false, MG_NETHER>(W, tree, states, ns, pts, np, out, tg, st);
        else points_t<false, MG_END>(W, tree, states, ns, pts, np, out, tg, st);
    }
    count_launch();
    return (int)cudaGetLastError();
}

int launch_density(const MgWorldDesc &W, const MgLattice *state, int n, const int32_t *xyz, double *out, cudaStream_t st) {
    if (n <= 0) return 0;
    if (W.dim != MG_OVERWORLD) return (int)cudaErrorInvalidValue;
    {
        ProfScope ps_(K_DENSITY, st);
        if (W.fmode) k_density<true><<<blocks_for(n, 128), 128, 0, st>>>(W, state, n, xyz, out);
        else k_density<false><<<blocks_for(n, 128), 128, 0, st>>>(W, state, n, xyz, out);
    }
    count_launch();
    return (int)cudaGetLastError();
}

template <bool FM, int DIM, bool CHAIN>
static void grid_t(const MgWorldDesc &W, const MgTreeNode *tree, const MgLattice *state, int qx0, int qz0, int nx, int nz,
                   int qy, uint8_t *out, ChainRec *rec, cudaStream_t st) {
    size_t sm = grid_smem_k(W);
    cudaFuncSetAttribute(k_grid<FM, DIM, CHAIN>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    const long long tiles = (long long)((nx + 7) / 8) * ((nz + 15) / 16);
    { ProfScope ps_(K_GRID, st); k_grid<FM, DIM, CHAIN><<<(unsigned)tiles, 128, sm, st>>>(W, tree, state, qx0, qz0, nx, nz, qy, out, rec); }
}
__global__ void k_end_lookup(const __grid_constant__ MgWorldDesc W, const uint8_t *__restrict__ cls, int cx0, int cz0,
                             int ncx, int qx0, int qz0, int nx, int nz, uint8_t *__restrict__ out) {
    const long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= (long long)nx * nz) return;
    int qx = qx0 + (int)(g % nx), qz = qz0 + (int)(g / nx);
    int cx = (qx * 4) >> 4, cz = (qz * 4) >> 4;
    out[g] = (uint8_t)W.end_ids[cls[(size_t)(cz - cz0) * ncx + (cx - cx0)]];
}
int launch_end_lookup(const MgWorldDesc &W, const uint8_t *cls, int cx0, int cz0, int ncx, int qx0, int qz0, int nx,
                      int nz, uint8_t *out, cudaStream_t st) {
    { ProfScope ps_(K_END_LOOKUP, st); k_end_lookup<<<blocks_for((long long)nx * nz, 256), 256, 0, st>>>(W, cls, cx0, cz0, ncx, qx0, qz0, nx, nz, out); }
    count_launch();
    return (int)cudaGetLastError();
}
size_t chain_scratch_bytes(long long ncells) { return (size_t)ncells * (sizeof(ChainRec) + sizeof(int32_t)); }
int launch_quart_grid(const MgWorldDesc &W, const MgTreeNode *tree, const MgLattice *state, int qx0, int qz0, int nx, int nz, int qy, int rule, uint8_t *out, void *scratch, cudaStream_t st) {
    long long n = (long long)nx * nz;
    if (n <= 0) return 0;
    if (W.dim == MG_END) {
        /* chunk classes over the grid's chunk range, then one lookup per cell */
        int cx0 = (qx0 * 4) >> 4, cz0 = (qz0 * 4) >> 4;
        int cx1 = ((qx0 + nx - 1) * 4) >> 4, cz1 = ((qz0 + nz - 1) * 4) >> 4;
        int ncx = cx1 - cx0 + 1, ncz = cz1 - cz0 + 1;
        uint8_t *cls = (uint8_t *)scratch;
        if (W.fmode) { ProfScope ps_(K_END_CHUNKS, st); k_end_chunks<true><<<end_tiles(ncx, ncz), 128, 0, st>>>(state, cx0, cz0, ncx, ncz, cls, W.end_f2, W.end_g2); }
        else { ProfScope ps_(K_END_CHUNKS, st); k_end_chunks<false><<<end_tiles(ncx, ncz), 128, 0, st>>>(state, cx0, cz0, ncx, ncz, cls, W.end_f2, W.end_g2); }
        count_launch();
        return launch_end_lookup(W, cls, cx0, cz0, ncx, qx0, qz0, nx, nz, out, st);
    }
    bool chain = rule == MG_TIE_GRID_CHAIN || rule == MG_TIE_CHUNK_ORDER;
    ChainRec *rec = (ChainRec *)scratch;
    if (W.fmode) {
        if (W.dim == MG_OVERWORLD) {
            if (chain) grid_t<true, MG_OVERWORLD, true>(W, tree, state, qx0, qz0, nx, nz, qy, out, rec, st);
            else grid_t<true, MG_OVERWORLD, false>(W, tree, state, qx0, qz0, nx, nz, qy, out, rec, st);
        } else {
            if (chain) grid_t<true, MG_NETHER, true>(W, tree, state, qx0, qz0, nx, nz, qy, out, rec, st);
            else grid_t<true, MG_NETHER, false>(W, tree, state, qx0, qz0, nx, nz, qy, out, rec, st);
        }
    } else {
        if (W.dim == MG_OVERWORLD) {
            if (chain) grid_t<false, MG_OVERWORLD, true>(W, tree, state, qx0, qz0, nx, nz, qy, out, rec, st);
            else grid_t<false, MG_OVERWORLD, false>(W, tree, state, qx0, qz0, nx, nz, qy, out, rec, st);
        } else {
            if (chain) grid_t<false, MG_NETHER, true>(W, tree, state, qx0, qz0, nx, nz, qy, out, rec, st);
            else grid_t<false, MG_NETHER, false>(W, tree, state, qx0, qz0, nx, nz, qy, out, rec, st);
        }
    }
    count_launch();
    if (rule == MG_TIE_GRID_CHAIN) {
        { ProfScope ps_(K_CHAIN_RESOLVE, st); k_chain_resolve<<<blocks_for(n, 256), 256, 0, st>>>(tree, rec, n, out); }
        count_launch();
    } else if (rule == MG_TIE_CHUNK_ORDER) {
        int32_t *order = reinterpret_cast<int32_t *>(rec + n);
        { ProfScope ps_(K_CHAIN_RESOLVE, st); k_chain_order<<<blocks_for(n, 256), 256, 0, st>>>(qx0, qz0, nx, nz, order); }
        count_launch();
        { ProfScope ps_(K_CHAIN_RESOLVE, st); k_chain_resolve_ordered<<<blocks_for(n, 256), 256, 0, st>>>(tree, rec, n, order, out); }
        count_launch();
    }
    return (int)cudaGetLastError();
}

template <bool FM, int DIM>
static void blockgrid_t(const MgWorldDesc &W, const MgTreeNode *tree, const MgLattice *state, int64_t zseed, int x0,
                        int z0, int nx, int nz, int step, int y, const int32_t *xyz, uint8_t *out, const uint8_t *cls,
                        int ecx0, int ecz0, int encx, cudaStream_t st) {
    size_t sm = DIM == MG_END ? 0 : grid_smem(W);
    if (sm) cudaFuncSetAttribute(k_blockgrid<FM, DIM>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    ProfScope ps_(K_BLOCKGRID, st);
    /* the kernel's warp-tile form (its own test of the same condition): one CTA per 16 x 8-cell tile */
    const bool tiles = FM && DIM == MG_OVERWORLD && !xyz && step <= 16 && W.tree_fanout >= MG_WARP_TREE_FANOUT;
    const unsigned nb = tiles ? (unsigned)(((long long)(nx + 15) / 16) * ((nz + 7) / 8)) : blocks_for((long long)nx * nz, 128);
    k_blockgrid<FM, DIM><<<nb, 128, sm, st>>>(W, tree, state, zseed, x0, z0, nx, nz, step, y, xyz, out, cls, ecx0, ecz0,
                                              encx);
}
/* Block-coordinate biomes: a grid (xyz == nullptr) or n = nx points (nz == 1) at xyz. For the End,
 * `scratch` holds the chunk classes of [ecx0, ecx0+encx) x [ecz0, ecz0+encz). */
int launch_block_biomes(const MgWorldDesc &W, const MgTreeNode *tree, const MgLattice *state, int64_t zseed, int x0,
                        int z0, int nx, int nz, int step, int y, const int32_t *xyz, uint8_t *out, void *scratch,
                        int ecx0, int ecz0, int encx, int encz, cudaStream_t st) {
    if ((long long)nx * nz <= 0) return 0;
    uint8_t *cls = (uint8_t *)scratch; /* End chunk classes, or null: evaluate per sample */
    if (W.dim == MG_END && cls) {
        if (W.fmode) { ProfScope ps_(K_END_CHUNKS, st); k_end_chunks<true><<<end_tiles(encx, encz), 128, 0, st>>>(state, ecx0, ecz0, encx, encz, cls, W.end_f2, W.end_g2); }
        else { ProfScope ps_(K_END_CHUNKS, st); k_end_chunks<false><<<end_tiles(encx, encz), 128, 0, st>>>(state, ecx0, ecz0, encx, encz, cls, W.end_f2, W.end_g2); }
        count_launch();
    }
    if (W.fmode) {
        if (W.dim == MG_OVERWORLD) blockgrid_t<true, MG_OVERWORLD>(W, tree, state, zseed, x0, z0, nx, nz, step, y, xyz, out, cls, ecx0, ecz0, encx, st);
        else if (W.dim == MG_NETHER) blockgrid_t<true, MG_NETHER>(W, tree, state, zseed, x0, z0, nx, nz, step, y, xyz, out, cls, ecx0, ecz0, encx, st);
        else blockgrid_t<true, MG_END>(W, tree, state, zseed, x0, z0, nx, nz, step, y, xyz, out, cls, ecx0, ecz0, encx, st);
    } else {
        if (W.dim == MG_OVERWORLD) blockgrid_t<false, MG_OVERWORLD>(W, tree, state, zseed, x0, z0, nx, nz, step, y, xyz, out, cls, ecx0, ecz0, encx, st);
        else if (W.dim == MG_NETHER) blockgrid_t<false, MG_NETHER>(W, tree, state, zseed, x0, z0, nx, nz, step, y, xyz, out, cls, ecx0, ecz0, encx, st);
        else blockgrid_t<false, MG_END>(W, tree, state, zseed, x0, z0, nx, nz, step, y, xyz, out, cls, ecx0, ecz0, encx, st);
    }
    count_launch();
    return (int)cudaGetLastError();
}

}  // namespace mg
