/* selfcheck.cu -- on-device check that the exact integer coordinate split (split_fk / split_dk) equals the
 * reference arithmetic (split_*_plain: (x * f) wrapped, + offset, floor, fraction, in double) bit for bit,
 * on generated inputs that cover the ranges the biome path sees and the edges of the fast path:
 * integer quart coordinates, coordinates plus a float shift, their products with the second-stack factor,
 * tiny and huge values, values whose sum with the offset lands near an integer, in (-1, 0) or on 0, and
 * offsets at 0, near 256 and on integers.  Also: the double branch's fixed-point octave (octave_dfix)
 * against the plain double octave on random permutations and fractions, the single-precision screen of
 * BiomeManager's zoom (zoom_pick) against the double-precision choice among all 8 candidates, the
 * fixed-point screen of the double branch's climate noises (nn_q + cast_settled_q) against the exact double
 * evaluation on a world's own seed lattices, and the double branch's whole Overworld climate as the kernels
 * compute it (climate_ow_d) against the plain double evaluation, and the 32-bit R-tree searches against
 * the 64-bit stack searches. */
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include "../../include/mcgen.h"
#include "abi_internal.h"
#include "climate.cuh"

using namespace mgd;

namespace {

__device__ __forceinline__ uint64_t mix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ULL;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

__global__ void k_check_split(long long n, uint64_t seed, unsigned long long *bad) {
    unsigned long long bf = 0, bd = 0;
    for (long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x; g < n; g += (long long)gridDim.x * blockDim.x) {
        uint64_t r0 = mix64(seed ^ (uint64_t)g), r1 = mix64(r0), r2 = mix64(r1), r3 = mix64(r2);
        const int k = (int)(r0 % 13) - 12;
        const double f = ldexp(1.0, k);
        double off;
        switch ((r1 >> 8) % 8) {
        case 0: off = 0.0; break;
        case 1: off = 255.99999999999997; break;
        case 2: off = (double)(r1 % 256); break;
        case 3: off = 0.5; break;
        default: off = (double)(r1 >> 11) * 0x1.0p-53 * 256.0; break;
        }
        double x;
        const int64_t sr = (int64_t)r2;
        switch (r0 >> 60) {
        case 0: x = (double)(sr >> 39); break;                               /* |x| < 2^24, integer */
        case 1: x = (double)(sr % 301); break;                               /* small integer */
        case 2: x = (double)(sr % 40000) + (double)(float)((double)(int32_t)r3 * 0x1.0p-27); break; /* + float shift */
        case 3: x = ((double)(sr % 3000000) + (double)(float)((double)(int32_t)r3 * 0x1.0p-28)) * MG_SECOND_STACK; break;
        case 4: x = ldexp((double)(r3 >> 11), -(int)(r2 % 120) - 20) * ((r2 >> 63) ? -1.0 : 1.0); break; /* tiny */
        case 5: { /* x * f + off near an integer, in (-1, 0) or on 0 */
            const double target = (double)((int)(r3 % 11) - 5) + ((r3 >> 40) % 3 == 0 ? 0.0 : ldexp((double)(int64_t)(r2 >> 50) - 8192.0, -(int)((r3 >> 20) % 60)));
            x = (target - off) / f;
            break;
        }
        case 6: x = ldexp((double)(r3 >> 11) * 0x1.0p-53 + 1.0, 20 + (int)(r2 % 8)) * ((r2 >> 62) & 1 ? -1.0 : 1.0); break; /* huge */
        case 7: x = -(double)(sr >> 40) - off / f; break;                     /* negative, sum near -integer */
        case 8: x = (double)(sr >> 42) + 0.25 * (double)(r3 % 4); break;
        default: x = ldexp((double)(int64_t)(r3 >> 10) * 0x1.0p-53, (int)(r2 % 56) - 30); break;
        }
        int ia, ib;
        float fa, fb;
        split_fk(x, f, k, off, ia, fa);
        split_f_plain(x * f, off, ib, fb);
        bf += (ia != ib) || (__float_as_uint(fa) != __float_as_uint(fb));
        double da, db;
        int64_t F;
        split_dk(x, f, k, off, ia, da, F);
        split_d_plain(x * f, off, ib, db);
        bd += (ia != ib) || (__double_as_longlong(da) != __double_as_longlong(db)) || F != fixed52(db);
        /* the multiply-high modulo of the legacy shuffles, against the division */
        {
            const int32_t d = 2 + (int32_t)(r3 % 255), u = (int32_t)(r2 >> 33);
            bd += mod_small(u, d) != u % d;
        }
    }
    if (bf) atomicAdd(&bad[0], bf);
    if (bd) atomicAdd(&bad[1], bd);
}

/* fixed-point double octave vs the plain double octave: random permutation per thread, fractions that are
 * multiples of 2^-52 (any, near 0, near 1, on small dyadic grids); equal as doubles (the sign of an exact
 * zero may differ, and is never observed downstream) */
__global__ void k_check_octave(long long n, uint64_t seed, unsigned long long *bad) {
    __shared__ uint8_t perm[128][256];
    uint8_t *P = perm[threadIdx.x];
    uint64_t r = mix64(seed ^ (0xC0FFEEULL + blockIdx.x * 977ULL + threadIdx.x));
    for (int i = 0; i < 256; i++) P[i] = (uint8_t)i;
    for (int i = 255; i > 0; i--) {
        r = mix64(r);
        const int j = (int)(r % (uint64_t)(i + 1));
        const uint8_t t = P[i]; P[i] = P[j]; P[j] = t;
    }
    const PlainPerm pp{P};
    unsigned long long b = 0;
    for (long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x; g < n; g += (long long)gridDim.x * blockDim.x) {
        int64_t F[3];
        for (int c = 0; c < 3; c++) {
            r = mix64(r ^ (uint64_t)g);
            switch (r >> 61) {
            case 0: F[c] = 0; break;
            case 1: F[c] = (int64_t)((r >> 8) & 0xFFF); break;                          /* near 0 */
            case 2: F[c] = (1LL << 52) - 1 - (int64_t)((r >> 8) & 0xFFF); break;        /* near 1 */
            case 3: F[c] = (int64_t)(((r >> 8) & 0xFF) << 44); break;                   /* dyadic grid */
            default: F[c] = (int64_t)((r >> 8) & ((1ULL << 52) - 1)); break;
            }
        }
        const int ix = (int)(r & 255) - 128, iy = (int)((r >> 8) & 255), iz = (int)((r >> 16) & 1023) - 512;
        const double fx = (double)F[0] * 0x1.0p-52, fy = (double)F[1] * 0x1.0p-52, fz = (double)F[2] * 0x1.0p-52;
        const double v = fade<double>(fy), w = fade<double>(fz);
        const double a = octave_dfix(pp, ix, fx, F[0], iy, F[1], v, iz, F[2], w);
        const double c = octave_q<double>(pp, ix, fx, iy, fy, fy - 1.0, v, iz, fz, fz - 1.0, w);
        b += !(a == c);
    }
    if (b) atomicAdd(bad, b);
}

/* zoom: random zoom seeds and block positions (|x|, |z| < 2^25, y in [-64, 320)); every case compares the
 * screened choice with the first strict minimum of the 8 double-precision distances (region.c:61-85) */
__global__ void k_check_zoom(long long n, uint64_t seed, unsigned long long *out) {
    unsigned long long bad = 0, close = 0;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const uint64_t r = mix64(seed ^ mix64((uint64_t)i)), r2 = mix64(r);
        const int64_t zseed = (int64_t)mix64(seed + (uint64_t)(i >> 10)); /* 1024 positions per zoom seed */
        const int x = (int)(r & 0x3FFFFFF) - (1 << 25), z = (int)((r >> 26) & 0x3FFFFFF) - (1 << 25);
        const int y = (int)(r2 % 384) - 64;
        const int ax = x - 2, ay = y - 2, az = z - 2;
        const int px = ax >> 2, py = ay >> 2, pz = az >> 2;
        int c;
        const int got = mg::zoom_pick(zseed, px, py, pz, ax & 3, ay & 3, az & 3, c);
        close += c > 1;
        double bd = __longlong_as_double(0x7FF0000000000000LL);
        int want = 0;
        for (int k = 0; k < 8; k++) {
            const int ox = (k >> 2) & 1, oy = (k >> 1) & 1, oz = k & 1;
            const double d = mg::zoom_dist_d(mg::zoom_draws(zseed, px + ox, py + oy, pz + oz),
                                             (ax & 3) / 4.0 - ox, (ay & 3) / 4.0 - oy, (az & 3) / 4.0 - oz);
            if (bd > d) { want = k; bd = d; }
        }
        bad += got != want;
    }
    atomicAdd(&out[0], bad);
    atomicAdd(&out[1], close);
}

/* noise screen: coordinates x = X + s with X an integer of magnitude class 2^10, 2^16, 2^21 or 2^25 and s a
 * random double in (-4, 4) (the climate noises take quart coordinates plus a shift of up to 4); every
 * screened noise of the world (Overworld: temperature .. ridge and ridges_folded; Nether: temperature,
 * vegetation) is compared with the float of the exact double value.  out: mismatches, cases the screen left
 * to the exact path, and the largest |fixed - exact| / fix_err as a double's bits. */
__global__ void k_check_noise(const __grid_constant__ MgWorldDesc W, const MgLattice *__restrict__ T, long long n,
                              uint64_t seed, unsigned long long *out) {
    unsigned long long bad = 0, left = 0;
    double worst = 0.0;
    const int nn = W.dim == MG_OVERWORLD ? 5 : 2;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const uint64_t r = mix64(seed ^ mix64((uint64_t)i)), r2 = mix64(r), r3 = mix64(r2), r4 = mix64(r3);
        const int lim = 1 << ((r & 3) == 0 ? 10 : ((r & 3) == 1 ? 16 : ((r & 3) == 2 ? 21 : 25)));
        const int X = (int)((r >> 8) % (uint64_t)(2 * lim)) - lim, Z = (int)((r2 >> 8) % (uint64_t)(2 * lim)) - lim;
        const double sx = ((double)(r3 >> 11) * 0x1.0p-53 * 2.0 - 1.0) * 4.0;
        const double sz = ((double)(r4 >> 11) * 0x1.0p-53 * 2.0 - 1.0) * 4.0;
        const double x = (double)X + sx, z = (double)Z + sz;
        const double xc = x * MG_SECOND_STACK, zc = z * MG_SECOND_STACK;
        for (int j = 0; j < nn; j++) {
            const MgNoise &N = W.dim == MG_OVERWORLD ? W.noise[1 + j] : W.nether[j];
            if (N.fix_err < 0.0) continue;
            const double e = mgd::nn_d_y0(N, T, x, z, xc, zc);
            float f;
            const int64_t q = mgd::nn_q<false>(N, T, x, z, xc, zc);
            if (q == MG_QFAIL) { left++; continue; }
            const double a = (double)q * 0x1.0p-59;
            const double ratio = fabs(a - e) / N.fix_err;
            worst = ratio > worst ? ratio : worst;
            if (!mgd::cast_settled_q(q, N.fix_eq, f)) { left++; continue; }
            bad += f != (float)e;
            if (W.dim == MG_OVERWORLD && j == 4) {
                const double rfe = (fabs(fabs(e) + W.rf_d[0]) + W.rf_d[1]) * W.rf_d[2];
                if (W.rf_eq < 0 || !mg::ridges_folded_settled(W, q, f)) { left++; continue; }
                bad += f != (float)rfe;
            }
        }
    }
    atomicAdd(&out[0], bad);
    atomicAdd(&out[1], left);
    atomicMax(&out[2], (unsigned long long)__double_as_longlong(worst)); /* non-negative: bits order as values */
}

/* 32-bit screen of the noises whose value is only quantised (the Nether kernels' form for their two noises;
 * the Overworld's temperature and vegetation, with other constants, are checked too), on k_check_noise's
 * coordinates: the screen's value against the exact double value.  out: targets
 * that differ from quantize((float)exact) where the screen settles them, values it leaves to the 59-bit
 * screen, the largest |value - exact| / bound as a double's bits, and the settled values whose exact value
 * lies within twice the bound of a target boundary (the cases that try the screen's margin). */
__global__ void k_check_noise_quant(const __grid_constant__ MgWorldDesc W, const MgLattice *__restrict__ T, long long n,
                                    uint64_t seed, unsigned long long *out) {
    unsigned long long bad = 0, left = 0, near = 0;
    double worst = 0.0;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const uint64_t r = mix64(seed ^ mix64((uint64_t)i)), r2 = mix64(r), r3 = mix64(r2), r4 = mix64(r3);
        const int lim = 1 << ((r & 3) == 0 ? 10 : ((r & 3) == 1 ? 16 : ((r & 3) == 2 ? 21 : 25)));
        const int X = (int)((r >> 8) % (uint64_t)(2 * lim)) - lim, Z = (int)((r2 >> 8) % (uint64_t)(2 * lim)) - lim;
        const double sx = ((double)(r3 >> 11) * 0x1.0p-53 * 2.0 - 1.0) * 4.0;
        const double sz = ((double)(r4 >> 11) * 0x1.0p-53 * 2.0 - 1.0) * 4.0;
        const double x = (double)X + sx, z = (double)Z + sz;
        const double xc = x * MG_SECOND_STACK, zc = z * MG_SECOND_STACK;
        for (int j = 0; j < 2; j++) {
            const MgNoise &N = W.dim == MG_OVERWORLD ? W.noise[1 + j] : W.nether[j];
            if (N.fix_eq32 < 0) continue;
            const double e = mgd::nn_d_y0(N, T, x, z, xc, zc);
            const int64_t q = mgd::nn_q32(N, T, x, z, xc, zc);
            if (q == MG_QFAIL) { left++; continue; }
            const double bound = (double)N.fix_eq32 * 0x1.0p-59;
            const double ratio = fabs((double)q * 0x1.0p-59 - e) / bound;
            worst = ratio > worst ? ratio : worst;
            float f;
            if (!mg::quant_settled_q(q, N.fix_eq32, f)) { left++; continue; }
            const int want = mgd::quantize((float)e);
            bad += mgd::quantize(f) != want;
            /* the exact value's distance to the nearest target boundary, in the float domain */
            const int64_t e59 = (int64_t)(e * 0x1.0p59);
            float g;
            near += !mg::quant_settled_q(e59, 2 * N.fix_eq32, g);
        }
    }
    atomicAdd(&out[0], bad);
    atomicAdd(&out[1], left);
    atomicMax(&out[2], (unsigned long long)__double_as_longlong(worst));
    atomicAdd(&out[3], near);
}

/* Overworld climate of the double branch as the kernels compute it (climate_ow_d: exact shift noises, the
 * five climate noises screened in fixed point) against the plain double evaluation of every noise: random
 * quart cells (|qx|, |qz| below 2^8, 2^11, 2^13, 2^15, 2^18 or 2^21, qy in [-16, 80)).  out: cells whose
 * six targets differ, cells with at least one value the screen left to the exact path. */
__global__ void k_check_climate(const __grid_constant__ MgWorldDesc W, const MgLattice *__restrict__ T, long long n,
                                uint64_t seed, unsigned long long *out) {
    unsigned long long bad = 0, left = 0;
    const int lims[6] = {8, 11, 13, 15, 18, 21};
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const uint64_t r = mix64(seed ^ mix64((uint64_t)i)), r2 = mix64(r), r3 = mix64(r2);
        const int lim = 1 << lims[(r & 0xFF) % 6];
        const int qx = (int)((r >> 8) % (uint64_t)(2 * lim)) - lim, qz = (int)((r2 >> 8) % (uint64_t)(2 * lim)) - lim;
        const int by = 4 * ((int)(r3 % 96) - 16);
        const double X = (double)qx, Z = (double)qz, Xc = X * MG_SECOND_STACK, Zc = Z * MG_SECOND_STACK;
        int32_t got[6], want[6];
        mg::climate_ow_d(W, W.spline, T, X, Z, Xc, Zc, by, got);
        const double x = X + mgd::nn_d_y0(W.noise[0], T, X, Z, Xc, Zc) * 4.0;
        const double z = Z + mgd::nn_d_z0(W.noise[0], T, Z, X, Zc, Xc) * 4.0;
        const double xc = x * MG_SECOND_STACK, zc = z * MG_SECOND_STACK;
        double v[5];
        bool exact = false;
        for (int j = 0; j < 5; j++) {
            const MgNoise &N = W.noise[1 + j];
            v[j] = mgd::nn_d_y0(N, T, x, z, xc, zc);
            const int64_t q = N.fix_err < 0.0 ? MG_QFAIL : mgd::nn_q<false>(N, T, x, z, xc, zc);
            float f;
            exact |= q == MG_QFAIL || !mgd::cast_settled_q(q, N.fix_eq, f);
            if (j == 4 && !exact) exact |= W.rf_eq < 0 || !mg::ridges_folded_settled(W, q, f);
        }
        mg::climate_finish_d(W, W.spline, v[0], v[1], v[2], v[3], v[4], by, want);
        bool diff = false;
        for (int j = 0; j < 6; j++) diff |= got[j] != want[j];
        bad += diff;
        left += exact;
    }
    atomicAdd(&out[0], bad);
    atomicAdd(&out[1], left);
}

/* R-tree searches: the level-unrolled and single-loop 32-bit searches (ENGINE rule) and the unrolled tie
 * search against the 64-bit stack searches, on random targets: quantised climate values in [-12000, 12000]
 * (the tables' range) for half of the cases, in [-40000, 40000] (beyond the 32-bit clamp, where the exact
 * 64-bit search must take over) for the other half, and neighbours of the previous case's target (small
 * moves, many ties) for a quarter.  out: differing leaves, differing fitness or tie flags. */
__global__ void k_check_tree(const MgTreeNode *__restrict__ T, long long n, uint64_t seed, unsigned long long *out) {
    unsigned long long bad_leaf = 0, bad_other = 0;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        uint64_t r = mix64(seed ^ mix64((uint64_t)i));
        const int range = (r & 1) ? 40000 : 12000;
        const bool near = ((r >> 1) & 3) == 0;
        int32_t t[6];
        for (int k = 0; k < 6; k++) {
            r = mix64(r);
            t[k] = near ? (int32_t)(r % 2001) - 1000 + (int32_t)((r >> 20) % 7) * 1500 - 4500
                        : (int32_t)(r % (uint64_t)(2 * range + 1)) - range;
        }
        uint64_t d0, d1, d2, d3, d4;
        bool tie0, tie1;
        const int l0 = mgd::tree_search_stack(T, t, -1, d0);
        const int l1 = mgd::tree_search(T, t, -1, d1);
        const int l2 = mgd::tree_search_scattered(T, t, -1, d2);
        const int l3 = mgd::tree_search_tie_stack(T, t, d3, tie0);
        const int l4 = mgd::tree_search_tie(T, t, d4, tie1);
        bad_leaf += (l1 != l0) + (l2 != l0) + (l3 != l0) + (l4 != l0);
        bad_other += (d1 != d0) + (d2 != d0) + (d3 != d0) + (d4 != d0) + (tie0 != tie1);
    }
    atomicAdd(&out[0], bad_leaf);
    atomicAdd(&out[1], bad_other);
}

/* The warp-shared search (tree_search_warp) against the 64-bit stack search on targets of the kind a warp of
 * neighbouring cells has: per warp a centre in the tables' range and per lane a spread of 50, 400, 2,000 or
 * 6,000 around it; about one lane in eight inactive; in one warp in sixteen one lane far outside the packed
 * range (the warp's fallback).  Case i is lane i % 32 of warp case i / 32.  out[0]: differing leaves. */
__global__ void __launch_bounds__(128) k_check_tree_warp(const MgTreeNode *__restrict__ T, long long n, uint64_t seed,
                                                         unsigned long long *out) {
    __shared__ WarpTreeScratch ws[4];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    unsigned long long bad = 0;
    const long long nw = (n + 31) / 32, step = (long long)gridDim.x * 4;
    for (long long wc = (long long)blockIdx.x * 4 + wib; wc < nw; wc += step) {
        uint64_t r = mix64(seed ^ mix64(0x5157ULL ^ (uint64_t)wc));
        const int spreads[4] = {50, 400, 2000, 6000};
        const int spread = spreads[r & 3];
        const bool far_lane = ((r >> 2) & 15) == 0 && lane == 7;
        uint64_t q = mix64(r ^ (uint64_t)(lane + 1) * 0x9E3779B97F4A7C15ULL);
        const bool active = wc * 32 + lane < n && (q & 7) != 0;
        int32_t t[6];
        for (int k = 0; k < 6; k++) {
            r = mix64(r);
            q = mix64(q);
            const int32_t c = (int32_t)(r % 24001) - 12000;
            t[k] = far_lane ? (int32_t)(q % 80001) - 40000 : c + (int32_t)(q % (uint64_t)(2 * spread + 1)) - spread;
        }
        const int lw = tree_search_warp(T, t, active, ws[wib]);
        if (active) {
            uint64_t d;
            bad += lw != tree_search_stack(T, t, -1, d);
        }
    }
    atomicAdd(&out[0], bad);
}

/* The End's screened island test (end_island) against the reference's double simplex: each CTA shuffles a
 * random permutation (java.util.Random style, thread 0), then its threads test cells at chunk-cell coordinates
 * of magnitude up to 2^7, 2^11, 2^15 or 2^21, both branches.  out: wrong decisions, cases the screen left to
 * the exact path, and the largest |float evaluation - double value| / END_ISLAND_E as double bits. */
__global__ void __launch_bounds__(128) k_check_end(long long n, uint64_t seed, double F2, double G2,
                                                   unsigned long long *out) {
    __shared__ uint8_t perm[256];
    unsigned long long bad = 0, left = 0;
    double worst = 0.0;
    const long long per_round = (long long)gridDim.x * blockDim.x * 64;
    for (long long base = 0; base < n; base += per_round) {
        __syncthreads();
        if (threadIdx.x == 0) {
            uint64_t r = mix64(seed ^ mix64((uint64_t)(base / per_round) * 0x9E37ULL + blockIdx.x));
            for (int k = 0; k < 256; k++) perm[k] = (uint8_t)k;
            for (int k = 255; k > 0; k--) {
                r = mix64(r);
                const int m = (int)(r % (uint64_t)(k + 1));
                const uint8_t a = perm[k];
                perm[k] = perm[m];
                perm[m] = a;
            }
        }
        __syncthreads();
        for (int q = 0; q < 64; q++) {
            const long long i = base + ((long long)blockIdx.x * blockDim.x + threadIdx.x) * 64 + q;
            if (i >= n) break;
            const uint64_t r = mix64(seed ^ mix64((uint64_t)i)), r2 = mix64(r);
            const int lims[4] = {7, 11, 15, 21};
            const int lim = 1 << lims[r & 3];
            const double x = (double)((long long)((r >> 8) % (uint64_t)(2 * lim)) - lim);
            const double z = (double)((long long)((r2 >> 8) % (uint64_t)(2 * lim)) - lim);
            const bool fm = (r >> 4) & 1;
            const double nv = mg::simplex2(perm, x, z, F2, G2);
            const bool exact = fm ? ((float)nv < -0.9f) : (nv < (double)-0.9f);
            bad += mg::end_island(perm, x, z, F2, G2, fm) != exact;
            /* the float evaluation alone, as end_island forms it, for the bound */
            const double s = (x + z) * F2;
            const int ci = mgd::ifloor(x + s), cj = mgd::ifloor(z + s);
            const double t = (double)(ci + cj) * G2;
            const double x0 = x - ((double)ci - t), y0 = z - ((double)cj - t);
            const int i1 = x0 > y0 ? 1 : 0, j1 = 1 - i1;
            const float g2 = (float)G2, xf = (float)x0, yf = (float)y0;
            const float xs[3] = {xf, xf - (float)i1 + g2, xf - 1.0f + 2.0f * g2};
            const float ys[3] = {yf, yf - (float)j1 + g2, yf - 1.0f + 2.0f * g2};
            const int ii = ci & 255, jj = cj & 255;
            const int gs[3] = {perm[(ii + perm[jj]) & 255] % 12, perm[(ii + i1 + perm[(jj + j1) & 255]) & 255] % 12,
                               perm[(ii + 1 + perm[(jj + 1) & 255]) & 255] % 12};
            float nf = 0.0f;
            for (int c = 0; c < 3; c++) {
                float tt = 0.5f - xs[c] * xs[c] - ys[c] * ys[c];
                if (tt > 0.0f) {
                    tt *= tt;
                    nf += tt * tt * mgd::gdot<float>(gs[c], xs[c], ys[c], 0.0f);
                }
            }
            nf *= 70.0f;
            worst = fmax(worst, fabs((double)nf - nv) / (double)END_ISLAND_E);
            left += !(nf < -0.9f - (END_ISLAND_E + 1e-4f) || nf >= -0.9f + (END_ISLAND_E + 1e-4f));
        }
    }
    atomicAdd(&out[0], bad);
    atomicAdd(&out[1], left);
    atomicMax(&out[2], (unsigned long long)__double_as_longlong(worst));
}

}  // namespace

extern "C" MCGEN_API int mcgen_gb300_check_end(long long n, unsigned long long seed, long long *bad, long long *screened_out,
                                               double *worst_ratio) {
    if (n < 0 || !bad || !screened_out || !worst_ratio) return MCGEN_E_ARG;
    std::lock_guard<std::mutex> lk(mg::abi_lock());
    if (!mg::abi_device_ready()) return MCGEN_E_UNSUPPORTED;
    unsigned long long *d = nullptr;
    if (cudaMalloc(&d, 3 * sizeof(unsigned long long)) != cudaSuccess) return MCGEN_E_NOMEM;
    cudaMemset(d, 0, 3 * sizeof(unsigned long long));
    const double F2 = 0.5 * (sqrt(3.0) - 1.0), G2 = (3.0 - sqrt(3.0)) / 6.0; /* the 2-D simplex skew and unskew */
    k_check_end<<<152 * 2, 128>>>(n, seed, F2, G2, d);
    unsigned long long h[3] = {0, 0, 0};
    cudaError_t e = cudaMemcpy(h, d, sizeof h, cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e != cudaSuccess) return MCGEN_E_INTERNAL;
    *bad = (long long)h[0];
    *screened_out = (long long)h[1];
    memcpy(worst_ratio, &h[2], sizeof(double));
    return MCGEN_OK;
}

extern "C" MCGEN_API int mcgen_gb300_check_tree(const McWorld *w, long long n, unsigned long long seed, long long *bad_leaf,
                                                long long *bad_other) {
    if (!w || n < 0 || !bad_leaf || !bad_other) return MCGEN_E_ARG;
    if (w->desc.dim == MG_END) return MCGEN_E_ARG; /* the End has no climate tree */
    std::lock_guard<std::mutex> lk(mg::abi_lock());
    if (!mg::abi_device_ready()) return MCGEN_E_UNSUPPORTED;
    int rc = mg::abi_world_device(const_cast<McWorld *>(w));
    if (rc) return rc;
    unsigned long long *d = nullptr;
    if (cudaMalloc(&d, 2 * sizeof(unsigned long long)) != cudaSuccess) return MCGEN_E_NOMEM;
    cudaMemset(d, 0, 2 * sizeof(unsigned long long));
    k_check_tree<<<152 * 4, 128>>>(w->d_tree, n, seed, d);
    k_check_tree_warp<<<152 * 4, 128>>>(w->d_tree, n, seed ^ 0xA5A5A5A5ULL, d);
    unsigned long long h[2] = {0, 0};
    cudaError_t e = cudaMemcpy(h, d, sizeof h, cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e != cudaSuccess) return MCGEN_E_INTERNAL;
    *bad_leaf = (long long)h[0];
    *bad_other = (long long)h[1];
    return MCGEN_OK;
}

extern "C" MCGEN_API int mcgen_gb300_check_climate(const McWorld *w, long long n, unsigned long long seed, long long *bad,
                                                   long long *fallback) {
    if (!w || n < 0 || !bad || !fallback) return MCGEN_E_ARG;
    if (w->desc.dim != MG_OVERWORLD || w->desc.fmode) return MCGEN_E_ARG; /* the double branch's Overworld only */
    std::lock_guard<std::mutex> lk(mg::abi_lock());
    if (!mg::abi_device_ready()) return MCGEN_E_UNSUPPORTED;
    int rc = mg::abi_world_device(const_cast<McWorld *>(w));
    if (rc) return rc;
    unsigned long long *d = nullptr;
    if (cudaMalloc(&d, 2 * sizeof(unsigned long long)) != cudaSuccess) return MCGEN_E_NOMEM;
    cudaMemset(d, 0, 2 * sizeof(unsigned long long));
    k_check_climate<<<152 * 4, 128>>>(w->desc, w->d_state, n, seed, d);
    unsigned long long h[2] = {0, 0};
    cudaError_t e = cudaMemcpy(h, d, sizeof h, cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e != cudaSuccess) return MCGEN_E_INTERNAL;
    *bad = (long long)h[0];
    *fallback = (long long)h[1];
    return MCGEN_OK;
}

extern "C" MCGEN_API int mcgen_gb300_check_noise_quant(const McWorld *w, long long n, unsigned long long seed,
                                                       long long *bad, long long *screened_out, double *worst_ratio,
                                                       long long *near_boundary) {
    if (!w || n < 0 || !bad || !screened_out || !worst_ratio || !near_boundary) return MCGEN_E_ARG;
    if (w->desc.dim == MG_END || w->desc.fmode) return MCGEN_E_ARG; /* the double branch's noises only */
    std::lock_guard<std::mutex> lk(mg::abi_lock());
    if (!mg::abi_device_ready()) return MCGEN_E_UNSUPPORTED;
    int rc = mg::abi_world_device(const_cast<McWorld *>(w));
    if (rc) return rc;
    unsigned long long *d = nullptr;
    if (cudaMalloc(&d, 4 * sizeof(unsigned long long)) != cudaSuccess) return MCGEN_E_NOMEM;
    cudaMemset(d, 0, 4 * sizeof(unsigned long long));
    k_check_noise_quant<<<152 * 4, 128>>>(w->desc, w->d_state, n, seed, d);
    unsigned long long h[4] = {0, 0, 0, 0};
    cudaError_t e = cudaMemcpy(h, d, sizeof h, cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e != cudaSuccess) return MCGEN_E_INTERNAL;
    *bad = (long long)h[0];
    *screened_out = (long long)h[1];
    memcpy(worst_ratio, &h[2], sizeof(double));
    *near_boundary = (long long)h[3];
    return MCGEN_OK;
}

extern "C" MCGEN_API int mcgen_gb300_check_noise(const McWorld *w, long long n, unsigned long long seed, long long *bad,
                                                 long long *screened_out, double *worst_ratio) {
    if (!w || n < 0 || !bad || !screened_out || !worst_ratio) return MCGEN_E_ARG;
    if (w->desc.dim == MG_END || w->desc.fmode) return MCGEN_E_ARG; /* the double branch's noises only */
    std::lock_guard<std::mutex> lk(mg::abi_lock());
    if (!mg::abi_device_ready()) return MCGEN_E_UNSUPPORTED;
    int rc = mg::abi_world_device(const_cast<McWorld *>(w));
    if (rc) return rc;
    unsigned long long *d = nullptr;
    if (cudaMalloc(&d, 3 * sizeof(unsigned long long)) != cudaSuccess) return MCGEN_E_NOMEM;
    cudaMemset(d, 0, 3 * sizeof(unsigned long long));
    k_check_noise<<<152 * 4, 128>>>(w->desc, w->d_state, n, seed, d);
    unsigned long long h[3] = {0, 0, 0};
    cudaError_t e = cudaMemcpy(h, d, sizeof h, cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e != cudaSuccess) return MCGEN_E_INTERNAL;
    *bad = (long long)h[0];
    *screened_out = (long long)h[1];
    memcpy(worst_ratio, &h[2], sizeof(double));
    return MCGEN_OK;
}

extern "C" MCGEN_API int mcgen_gb300_check_zoom(long long n, unsigned long long seed, long long *bad, long long *screened_out) {
    if (n < 0 || !bad || !screened_out) return MCGEN_E_ARG;
    unsigned long long *d = nullptr;
    if (cudaMalloc(&d, 2 * sizeof(unsigned long long)) != cudaSuccess) return MCGEN_E_NOMEM;
    cudaMemset(d, 0, 2 * sizeof(unsigned long long));
    k_check_zoom<<<152 * 4, 256>>>(n, seed, d);
    unsigned long long h[2] = {0, 0};
    cudaError_t e = cudaMemcpy(h, d, sizeof h, cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e != cudaSuccess) return MCGEN_E_INTERNAL;
    *bad = (long long)h[0];
    *screened_out = (long long)h[1];
    return MCGEN_OK;
}

extern "C" MCGEN_API int mcgen_gb300_check_octave(long long n, unsigned long long seed, long long *bad) {
    if (n < 0 || !bad) return MCGEN_E_ARG;
    unsigned long long *d = nullptr;
    if (cudaMalloc(&d, sizeof(unsigned long long)) != cudaSuccess) return MCGEN_E_NOMEM;
    cudaMemset(d, 0, sizeof(unsigned long long));
    k_check_octave<<<152 * 2, 128>>>(n, seed, d);
    unsigned long long h = 0;
    cudaError_t e = cudaMemcpy(&h, d, sizeof h, cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e != cudaSuccess) return MCGEN_E_INTERNAL;
    *bad = (long long)h;
    return MCGEN_OK;
}

extern "C" MCGEN_API int mcgen_gb300_check_split(long long n, unsigned long long seed, long long *bad_f, long long *bad_d) {
    if (n < 0 || !bad_f || !bad_d) return MCGEN_E_ARG;
    unsigned long long *d = nullptr;
    if (cudaMalloc(&d, 2 * sizeof(unsigned long long)) != cudaSuccess) return MCGEN_E_NOMEM;
    cudaMemset(d, 0, 2 * sizeof(unsigned long long));
    k_check_split<<<152 * 8, 256>>>(n, seed, d);
    unsigned long long h[2] = {0, 0};
    cudaError_t e = cudaMemcpy(h, d, sizeof h, cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e != cudaSuccess) return MCGEN_E_INTERNAL;
    *bad_f = (long long)h[0];
    *bad_d = (long long)h[1];
    return MCGEN_OK;
}
