/* fused.cu -- many seeds x fixed points, Overworld: k_ow_seed_climate + k_ow_finish_tree.
 *
 * One CTA owns S seeds and one thread owns one lattice of one seed (46 per Overworld seed).  A thread
 * shuffles its permutation in shared memory (interleaved layout: byte i of thread t in word [i >> 2][t],
 * so all of a thread's accesses hit bank t % 32) and then samples *its own* lattice at every point of its
 * seed -- the lattices never leave the SM and their lookups never conflict.  Per-lattice octave values go
 * to shared memory, and one thread per (seed, point) sums them in the reference's order
 * (engine/mc_noise.h:285-324), forms the shifted coordinates after the ShiftA/ShiftB pass
 * (engine/mc_climate.h:113-164) and writes the five noise values.  k_ow_finish_tree then finishes the
 * climate and searches the R-tree (ENGINE rule) with one thread per sample, at full occupancy: inside the
 * fused kernel that serial per-point work would leave most of a CTA idle at its barriers.
 *
 * Phases per chunk of NPC points:  B  offset lattices: ShiftA and ShiftB octaves
 *                                   C  (seed, point): shift sums -> shifted x, z
 *                                   D  climate lattices: octaves at the shifted coordinates
 *                                   E  (seed, point): noise sums -> clim
 */
#include <cuda_runtime.h>
#include <stdint.h>

#include <type_traits>

#include "climate.cuh"
#include "launch.h"
#include "search.cuh"
#include "prof.h"

namespace mg {

/* threads per CTA: 4 seeds x 46 lattices, no idle thread, so that the float branch's shared memory (55.9 KB:
 * 64 permutation rows of FPS words, the chunk's octave values, offset headers) fits 4 CTAs per SM; the
 * double branch's (63.3 KB, values in double) fits 3 */
#define FNT 184
/* words per permutation row: byte i of thread t's permutation is in word [i >> 2][t]; a row of a multiple of
 * 32 words puts every thread's bytes in bank t % 32 whatever the row, so the shuffle's random swaps never
 * conflict (with 184 words a swap's bank would depend on its row) */
#define FPS 192
#define FNPC 8  /* points per chunk */
#define FMAXT 48 /* lattices per seed this kernel supports */

#define FMAXS 4  /* seeds per CTA at 46 lattices per seed */
#define FMAXOFF 24 /* offset-noise lattices per CTA (6 per seed) */

/* header of an offset-noise lattice, shared so that any thread can sample it: all of it for the double
 * branch, the fields the float branch's octaves read (offsets, floors, zero-coordinate split) for the float */
struct OffHdr {
    double ox, oy, oz, fyd, fzd, uyd, uzd;
    int64_t Fy, Fz;
    int iy, iz;
    MgLatZero z0;
};
struct OffHdrF {
    double ox, oy, oz;
    int iy, iz;
    MgLatZero z0;
    __device__ OffHdrF &operator=(const OffHdr &h) {
        ox = h.ox; oy = h.oy; oz = h.oz; iy = h.iy; iz = h.iz; z0 = h.z0;
        return *this;
    }
};

template <typename V>
struct FusedSmem {
    uint32_t perm[64][FPS];
    V val[FNT][FNPC];               /* octave value of lattice (owner thread) t at point p of the chunk */
    union {                         /* valb until phase C has read it, then coord (phase C syncs between) */
        V valb[FMAXOFF][FNPC];      /* ShiftB octave of the offset lattices */
        double coord[FMAXS][FNPC][4]; /* per (seed, point): x, z, x*c, z*c */
    };
    typename std::conditional<std::is_same<V, float>::value, OffHdrF, OffHdr>::type hdr[FMAXOFF];
};

/* Threads are lattice-major: thread t owns lattice j = t / spc of local seed t % spc, so the offset-noise
 * lattices of all the CTA's seeds are threads 0 .. noff*spc-1 and their shift octaves (16 per point) can be
 * spread over every thread of the CTA in phase B. */
template <bool FM>
__global__ void __launch_bounds__(FNT) k_ow_seed_climate(const __grid_constant__ MgWorldDesc W,
                                                         const int64_t *__restrict__ seeds, int ns,
                                                         const int32_t *__restrict__ pts, int np, int pstride,
                                                         typename std::conditional<FM, float, double>::type *__restrict__ clim) {
    typedef typename std::conditional<FM, float, double>::type V;
    extern __shared__ uint4 smem_raw[];
    FusedSmem<V> &sm = *reinterpret_cast<FusedSmem<V> *>(smem_raw);
    const int t = threadIdx.x;
    const int nt = W.ntables;
    const int spc = FNT / nt;                 /* seeds per CTA */
    const int s0 = blockIdx.x * spc;          /* first seed of the CTA */
    const int j = t / spc, ls = t % spc;      /* lattice index, local seed */
    const bool active = j < nt && s0 + ls < ns;
    const MgNoise &O = W.noise[0];
    const int noff = 2 * O.nlev;              /* offset-noise lattices per seed (noise 0 is first) */
    const int nown = noff * spc;              /* offset-noise lattice owners in the CTA */

    /* ---- phase A: this thread's lattice (engine/mc_climate.h:95-106, engine/mc_noise.h:29-41) */
    int noise = 0, st = 0, lev = 0;
    double ox = 0.0, oy = 0.0, oz = 0.0;
    if (active) {
        while (noise < MG_OW_NOISES - 1 && j >= W.noise[noise + 1].base) noise++;
        const MgNoise &N = W.noise[noise];
        const int r = j - N.base;
        st = r >= N.nlev;
        lev = r - st * N.nlev;
        Xo root = xo_from_seed(seeds[s0 + ls]);
        uint64_t plo = xo_next(root), phi = xo_next(root);
        Xo nr = xo_make(W.nhl[noise] ^ plo, W.nhh[noise] ^ phi);
        uint64_t a = xo_next(nr), b = xo_next(nr);
        if (st) { a = xo_next(nr); b = xo_next(nr); }
        Xo x = xo_make(N.hlo[lev] ^ a, N.hhi[lev] ^ b);
        ox = xo_double(x) * 256.0;
        oy = xo_double(x) * 256.0;
        oz = xo_double(x) * 256.0;
        for (int w = 0; w < 64; w++) sm.perm[w][t] = 0x03020100u + 0x04040404u * (uint32_t)w;
        uint8_t *mine = reinterpret_cast<uint8_t *>(&sm.perm[0][t]); /* byte i at mine + (i>>2)*4*FPS + (i&3) */
        for (int qw = 0; qw < 64; qw++) {
#pragma unroll
            for (int r4 = 0; r4 < 4; r4++) {
                const int q = 4 * qw + r4;
                const int k = q + xo_int(x, 256u - (uint32_t)q);
                uint8_t *pa = mine + qw * (4 * FPS) + r4;
                uint8_t *pb = mine + (k >> 2) * (4 * FPS) + (k & 3);
                uint8_t va = *pa, vb = *pb;
                *pa = vb;
                *pb = va;
            }
        }
    }
    /* split of the offsets used by a zero input coordinate */
    OffHdr h;
    h.ox = ox; h.oy = oy; h.oz = oz;
    lattice_header(h, !FM);
    if (t < nown) sm.hdr[t] = h;
    const uint8_t *pbase = reinterpret_cast<const uint8_t *>(&sm.perm[0][0]);
    const MgNoise &N = W.noise[noise];
    const double f = N.freq[lev];
    const int fk = N.fexp[lev];

    for (int p0 = 0; p0 < np; p0 += FNPC) {
        const int npc = min(FNPC, np - p0);
        __syncthreads(); /* lattices and headers complete / previous chunk consumed */
        /* ---- phase B: ShiftA (x, 0, z) and ShiftB (z, x, 0) octaves, item = (owner, point) */
        for (int item = t; item < nown * npc; item += FNT) {
            const int o = item % nown, p = item / nown;
            const int oj = o / spc;
            const int ost = oj >= O.nlev, olev = oj - ost * O.nlev;
            if (s0 + o % spc >= ns) continue;
            const auto &oh = sm.hdr[o];
            const IlvPerm<FPS> perm{pbase, o};
            const int32_t *pp = pts + (size_t)(s0 + o % spc) * pstride + 3 * (p0 + p);
            double X = (double)pp[0], Z = (double)pp[2];
            if (ost) { X = X * MG_SECOND_STACK; Z = Z * MG_SECOND_STACK; }
            const double of = O.freq[olev];
            const int ok = O.fexp[olev];
            if constexpr (FM) {
                int ix, izz, iyy;
                float fx, fzz, fyy;
                split_fk(X, of, ok, oh.ox, ix, fx);
                split_fk(Z, of, ok, oh.oz, izz, fzz);
                sm.val[o][p] = (V)octave_y0<float>(perm, oh, ix, fx, izz, fzz);
                split_fk(Z, of, ok, oh.ox, ix, fx);
                split_fk(X, of, ok, oh.oy, iyy, fyy);
                sm.valb[o][p] = (V)octave_z0<float>(perm, oh, ix, fx, iyy, fyy);
            } else {
                int ix, izz, iyy;
                double fx, fzz, fyy;
                int64_t FX, FZ, FY;
                split_dk(X, of, ok, oh.ox, ix, fx, FX);
                split_dk(Z, of, ok, oh.oz, izz, fzz, FZ);
                sm.val[o][p] = (V)octave_d_y0(perm, oh, ix, fx, FX, izz, fzz, FZ);
                split_dk(Z, of, ok, oh.ox, ix, fx, FX);
                split_dk(X, of, ok, oh.oy, iyy, fyy, FY);
                sm.valb[o][p] = (V)octave_d_z0(perm, oh, ix, fx, FX, iyy, fyy, FY);
            }
        }
        __syncthreads();
        /* ---- phase C: shift sums and shifted coordinates, one thread per (seed, point) */
        double cx = 0.0, cz = 0.0;
        bool cw = false;
        if (t < spc * FNPC) {
            const int cs = t / FNPC, p = t % FNPC;
            if (p < npc && s0 + cs < ns) {
                const int32_t *pp = pts + (size_t)(s0 + cs) * pstride + 3 * (p0 + p);
                const double X = (double)pp[0], Z = (double)pp[2];
                double x, z;
                if (FM) {
                    float sa = 0.0f, sb = 0.0f;
                    for (int k = 0; k < O.nlev; k++) {
                        sa += O.amp_f[k] * (float)sm.val[k * spc + cs][p];
                        sa += O.amp_f[k] * (float)sm.val[(O.nlev + k) * spc + cs][p];
                    }
                    for (int k = 0; k < O.nlev; k++) {
                        sb += O.amp_f[k] * (float)sm.valb[k * spc + cs][p];
                        sb += O.amp_f[k] * (float)sm.valb[(O.nlev + k) * spc + cs][p];
                    }
                    x = X + (double)(sa * 4.0f);
                    z = Z + (double)(sb * 4.0f);
                } else {
                    double a1 = 0.0, a2 = 0.0, b1 = 0.0, b2 = 0.0;
                    for (int k = 0; k < O.nlev; k++) a1 += O.amp_d[k] * (double)sm.val[k * spc + cs][p] * O.vf_d[k];
                    for (int k = 0; k < O.nlev; k++) a2 += O.amp_d[k] * (double)sm.val[(O.nlev + k) * spc + cs][p] * O.vf_d[k];
                    for (int k = 0; k < O.nlev; k++) b1 += O.amp_d[k] * (double)sm.valb[k * spc + cs][p] * O.vf_d[k];
                    for (int k = 0; k < O.nlev; k++) b2 += O.amp_d[k] * (double)sm.valb[(O.nlev + k) * spc + cs][p] * O.vf_d[k];
                    x = X + ((a1 + a2) * O.vfac) * 4.0;
                    z = Z + ((b1 + b2) * O.vfac) * 4.0;
                }
                cx = x;
                cz = z;
                cw = true;
            }
        }
        __syncthreads(); /* every valb read is done: coord may overwrite it */
        if (cw) {
            const int cs = t / FNPC, p = t % FNPC;
            sm.coord[cs][p][0] = cx;
            sm.coord[cs][p][1] = cz;
            sm.coord[cs][p][2] = cx * MG_SECOND_STACK;
            sm.coord[cs][p][3] = cz * MG_SECOND_STACK;
        }
        __syncthreads();
        /* ---- phase D: climate octaves at (x, 0, z), each thread on its own lattice */
        if (active && noise != 0) {
            const IlvPerm<FPS> perm{pbase, t};
            for (int p = 0; p < npc; p++) {
                const double x = sm.coord[ls][p][st ? 2 : 0], z = sm.coord[ls][p][st ? 3 : 1];
                if (FM) {
                    int ix, izz;
                    float fx, fzz;
                    split_fk(x, f, fk, ox, ix, fx);
                    split_fk(z, f, fk, oz, izz, fzz);
                    sm.val[t][p] = (V)octave_y0<float>(perm, h, ix, fx, izz, fzz);
                } else {
                    int ix, izz;
                    double fx, fzz;
                    int64_t FX, FZ;
                    split_dk(x, f, fk, ox, ix, fx, FX);
                    split_dk(z, f, fk, oz, izz, fzz, FZ);
                    sm.val[t][p] = (V)octave_d_y0(perm, h, ix, fx, FX, izz, fzz, FZ);
                }
            }
        }
        __syncthreads();
        /* ---- phase E: the five noise sums of every (seed, point) -> clim[(s * np + p) * 5 + q] */
        if (t < spc * FNPC) {
            const int cs = t / FNPC, p = t % FNPC;
            if (p < npc && s0 + cs < ns) {
                V *dst = clim + ((size_t)(s0 + cs) * np + p0 + p) * 5;
                for (int q = 1; q < MG_OW_NOISES; q++) {
                    const MgNoise &Q = W.noise[q];
                    if (FM) {
                        float acc = 0.0f;
                        for (int k = 0; k < Q.nlev; k++) {
                            acc += Q.amp_f[k] * (float)sm.val[(Q.base + k) * spc + cs][p];
                            acc += Q.amp_f[k] * (float)sm.val[(Q.base + Q.nlev + k) * spc + cs][p];
                        }
                        dst[q - 1] = (V)acc;
                    } else {
                        double a1 = 0.0, a2 = 0.0;
                        for (int k = 0; k < Q.nlev; k++) a1 += Q.amp_d[k] * (double)sm.val[(Q.base + k) * spc + cs][p] * Q.vf_d[k];
                        for (int k = 0; k < Q.nlev; k++) a2 += Q.amp_d[k] * (double)sm.val[(Q.base + Q.nlev + k) * spc + cs][p] * Q.vf_d[k];
                        dst[q - 1] = (V)((a1 + a2) * Q.vfac);
                    }
                }
            }
        }
    }
}

/* Finish the climate of every sample from its five noise values (ridges_folded, offset spline, depth,
 * quantisation; engine/mc_climate.h:126-170) and search the R-tree (ENGINE rule). One thread per sample. */
template <bool FM>
__global__ void __launch_bounds__(128) k_ow_finish_tree(const __grid_constant__ MgWorldDesc W,
                                                        const MgTreeNode *__restrict__ tree,
                                                        const typename std::conditional<FM, float, double>::type *__restrict__ clim,
                                                        int ns, const int32_t *__restrict__ pts, int np, int pstride,
                                                        uint8_t *__restrict__ out, int32_t *__restrict__ targets) {
    __shared__ MgSpline S;
    {
        const uint4 *c = reinterpret_cast<const uint4 *>(&W.spline);
        uint4 *d = reinterpret_cast<uint4 *>(&S);
        for (int i = threadIdx.x; i < (int)(sizeof(MgSpline) / 16); i += blockDim.x) d[i] = c[i];
    }
    __syncthreads();
    const long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= (long long)ns * np) return;
    const int p = (int)(g % np);
    const int by = pts[(size_t)(g / np) * pstride + 3 * p + 1] * 4;
    int32_t tg[6];
    const auto *v = clim + (size_t)g * 5;
    if (FM) climate_finish_f(W, S, (float)v[0], (float)v[1], (float)v[2], (float)v[3], (float)v[4], by, tg);
    else climate_finish_d(W, S, (double)v[0], (double)v[1], (double)v[2], (double)v[3], (double)v[4], by, tg);
    uint64_t d;
    const int leaf = tree_search_scattered(tree, tg, -1, d);
    out[g] = tree[leaf].biome;
    if (targets)
        for (int k = 0; k < 6; k++) targets[g * 6 + k] = tg[k];
}

/* Seed search, Overworld, first observation of every candidate: finish the climate at the candidate's own
 * cell, check the observation (mask, or any equal-fitness leaf in ties mode); passing candidates are
 * appended to `surv`, failures counted into *fail (engine/cuda/mc_gpu.cuh:476-493, stage [0]). */
template <bool FM>
__global__ void __launch_bounds__(128) k_ow_search_first(const __grid_constant__ MgWorldDesc W,
                                                         const MgTreeNode *__restrict__ tree,
                                                         const typename std::conditional<FM, float, double>::type *__restrict__ clim,
                                                         int ns, const int64_t *__restrict__ seeds,
                                                         const int32_t *__restrict__ pts, MgObs o, int ties,
                                                         int64_t *__restrict__ surv, unsigned *__restrict__ nsurv,
                                                         unsigned long long *__restrict__ fail) {
    __shared__ MgSpline S;
    {
        const uint4 *c = reinterpret_cast<const uint4 *>(&W.spline);
        uint4 *d = reinterpret_cast<uint4 *>(&S);
        for (int i = threadIdx.x; i < (int)(sizeof(MgSpline) / 16); i += blockDim.x) d[i] = c[i];
    }
    __syncthreads();
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    bool failed = false;
    if (g < ns) {
        int32_t tg[6];
        const auto *v = clim + (size_t)g * 5;
        const int by = pts[3 * g + 1] * 4;
        if (FM) climate_finish_f(W, S, (float)v[0], (float)v[1], (float)v[2], (float)v[3], (float)v[4], by, tg);
        else climate_finish_d(W, S, (double)v[0], (double)v[1], (double)v[2], (double)v[3], (double)v[4], by, tg);
        if (obs_accept(o, tree, tg, ties != 0)) surv[atomicAdd(nsurv, 1u)] = seeds[g];
        else failed = true;
    }
    const int nf = __syncthreads_count(failed);
    if (threadIdx.x == 0 && nf) atomicAdd(fail, (unsigned long long)nf);
}

template <bool FM>
static int search_first_t(const MgWorldDesc &W, const MgTreeNode *tree, const int64_t *seeds, int ns, const int32_t *pts,
                          const MgObs &o, int ties, void *scratch, int64_t *surv, unsigned *nsurv,
                          unsigned long long *fail, cudaStream_t st) {
    typedef typename std::conditional<FM, float, double>::type V;
    const size_t sm = sizeof(FusedSmem<V>);
    cudaError_t e = cudaFuncSetAttribute(k_ow_seed_climate<FM>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (!e) e = cudaFuncSetAttribute(k_ow_seed_climate<FM>, cudaFuncAttributePreferredSharedMemoryCarveout,
                                     (int)cudaSharedmemCarveoutMaxShared); /* room for 4 CTAs per SM */
    if (e) return (int)e;
    const int spc = FNT / W.ntables;
    V *clim = (V *)scratch;
    {
        ProfScope ps_(K_OW_SEED_CLIMATE, st);
        k_ow_seed_climate<FM><<<(unsigned)((ns + spc - 1) / spc), FNT, sm, st>>>(W, seeds, ns, pts, 1, 3, clim);
    }
    count_launch_external();
    {
        ProfScope ps_(K_SEARCH_FIRST, st);
        k_ow_search_first<FM><<<(unsigned)((ns + 127) / 128), 128, 0, st>>>(W, tree, clim, ns, seeds, pts, o, ties, surv,
                                                                             nsurv, fail);
    }
    count_launch_external();
    return 0;
}

int launch_ow_search_first(const MgWorldDesc &W, const MgTreeNode *tree, const int64_t *seeds, int ns, const int32_t *pts,
                           const MgObs &o, int ties, void *scratch, int64_t *surv, unsigned *nsurv,
                           unsigned long long *fail, cudaStream_t st) {
    if (ns <= 0) return 0;
    int rc = W.fmode ? search_first_t<true>(W, tree, seeds, ns, pts, o, ties, scratch, surv, nsurv, fail, st)
                     : search_first_t<false>(W, tree, seeds, ns, pts, o, ties, scratch, surv, nsurv, fail, st);
    return rc ? rc : (int)cudaGetLastError();
}

bool fused_supported(const MgWorldDesc &W) {
    if (W.dim != MG_OVERWORLD || W.ntables > FMAXT || W.noise[0].base != 0) return false;
    const int spc = FNT / W.ntables;
    return spc >= 1 && spc <= FMAXS && 2 * W.noise[0].nlev * spc <= FMAXOFF;
}
size_t fused_scratch_bytes(const MgWorldDesc &W, long long samples) {
    return (size_t)samples * 5 * (W.fmode ? sizeof(float) : sizeof(double));
}

template <bool FM>
static int fused_t(const MgWorldDesc &W, const MgTreeNode *tree, const int64_t *seeds, int ns, const int32_t *pts, int np,
                   uint8_t *out, int32_t *tg, void *scratch, cudaStream_t st) {
    typedef typename std::conditional<FM, float, double>::type V;
    const size_t sm = sizeof(FusedSmem<V>);
    cudaError_t e = cudaFuncSetAttribute(k_ow_seed_climate<FM>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (!e) e = cudaFuncSetAttribute(k_ow_seed_climate<FM>, cudaFuncAttributePreferredSharedMemoryCarveout,
                                     (int)cudaSharedmemCarveoutMaxShared); /* room for 4 CTAs per SM */
    if (e) return (int)e;
    const int spc = FNT / W.ntables;
    V *clim = (V *)scratch;
    {
        ProfScope ps_(K_OW_SEED_CLIMATE, st);
        k_ow_seed_climate<FM><<<(unsigned)((ns + spc - 1) / spc), FNT, sm, st>>>(W, seeds, ns, pts, np, 0, clim);
    }
    count_launch_external();
    const long long n = (long long)ns * np;
    {
        ProfScope ps_(K_OW_FINISH_TREE, st);
        k_ow_finish_tree<FM><<<(unsigned)((n + 127) / 128), 128, 0, st>>>(W, tree, clim, ns, pts, np, 0, out, tg);
    }
    count_launch_external();
    return 0;
}

int launch_ow_seed_points(const MgWorldDesc &W, const MgTreeNode *tree, const int64_t *seeds, int ns, const int32_t *pts,
                          int np, uint8_t *out, int32_t *tg, void *scratch, cudaStream_t st) {
    if ((long long)ns * np <= 0) return 0;
    int rc = W.fmode ? fused_t<true>(W, tree, seeds, ns, pts, np, out, tg, scratch, st)
                     : fused_t<false>(W, tree, seeds, ns, pts, np, out, tg, scratch, st);
    return rc ? rc : (int)cudaGetLastError();
}

}  // namespace mg
