/* climate.cuh -- climate, End island, zoom and chunk-cell functions of the biome path (device).
 *
 * Shared by the grid/point kernels (kernels.cu) and the fused many-seed kernel (fused.cu).
 */
#ifndef MG_CLIMATE_CUH
#define MG_CLIMATE_CUH
#include "device.cuh"

namespace mg {
using namespace mgd;

/* ============================================================================ climate */
/* ridges_folded, offset spline, y-clamped depth gradient and quantisation of the five noise values
 * (engine/mc_climate.h:126-170), float branch */
__device__ __forceinline__ void climate_finish_f(const MgWorldDesc &W, const MgSpline &S, float tv, float hv, float cv,
                                                 float ev, float rv, int by, int32_t tg[6]) {
    float a = fabsf(rv) + W.rf_f[0];
    float rf = (fabsf(a) + W.rf_f[1]) * W.rf_f[2];
    float co[4] = {cv, ev, rv, rf};
    float off = W.off_f + spline_eval(S, co);
    int lo = min(W.grad_from_y, W.grad_to_y), hi = max(W.grad_from_y, W.grad_to_y);
    int yy = by < lo ? lo : (by > hi ? hi : by);
    float depth = (W.grad_from_f + (float)(yy - W.grad_from_y) * W.grad_fac_f) + off;
    tg[0] = quantize(tv); tg[1] = quantize(hv); tg[2] = quantize(cv);
    tg[3] = quantize(ev); tg[4] = quantize(depth); tg[5] = quantize(rv);
}
/* the double branch's depth gradient at block y, clamped (y_clamped_gradient): a function of y alone, which
 * the tile kernels compute once per tile (an IEEE double division and conversions: about 20 FP64 operations) */
__device__ __forceinline__ double depth_grad_d(const MgWorldDesc &W, int by) {
    const double fac = ((double)by - (double)W.grad_from_y) / ((double)W.grad_to_y - (double)W.grad_from_y);
    return fac < 0.0 ? W.grad_from_d : (fac > 1.0 ? W.grad_to_d : W.grad_from_d + fac * (W.grad_to_d - W.grad_from_d));
}
/* the same in the double branch */
__device__ __forceinline__ void climate_finish_d(const MgWorldDesc &W, const MgSpline &S, double tv, double hv, double cv,
                                                 double ev, double rv, int by, int32_t tg[6]) {
    double rf = (fabs(fabs(rv) + W.rf_d[0]) + W.rf_d[1]) * W.rf_d[2];
    float co[4] = {(float)cv, (float)ev, (float)rv, (float)rf};
    double off = 0.0 + (W.off_d + (double)spline_eval(S, co)) * 1.0;
    double depth = depth_grad_d(W, by) + off;
    tg[0] = quantize((float)tv); tg[1] = quantize((float)hv); tg[2] = quantize((float)cv);
    tg[3] = quantize((float)ev); tg[4] = quantize((float)depth); tg[5] = quantize((float)rv);
}

/* the same from the float values the reference takes of the five noises and of ridges_folded, with the
 * depth gradient g = depth_grad_d(W, by) given */
__device__ __forceinline__ void climate_finish_df(const MgWorldDesc &W, const MgSpline &S, float tf, float hf, float cf,
                                                  float ef, float rvf, float rff, double g, int32_t tg[6]) {
    float co[4] = {cf, ef, rvf, rff};
    double off = 0.0 + (W.off_d + (double)spline_eval(S, co)) * 1.0;
    double depth = g + off;
    tg[0] = quantize(tf); tg[1] = quantize(hf); tg[2] = quantize(cf);
    tg[3] = quantize(ef); tg[4] = quantize((float)depth); tg[5] = quantize(rvf);
}
/* (float) of a double-branch NormalNoise at (x, 0, z): the screened fixed-point value when it settles the
 * rounding, else the exact double evaluation */
__device__ __forceinline__ float nn_d_y0_float(const MgNoise &N, const MgLattice *__restrict__ T, double x, double z,
                                               double xc, double zc) {
    float f;
    if (N.fix_eq >= 0) {
        const int64_t q = nn_q<false>(N, T, x, z, xc, zc);
        if (q != MG_QFAIL && cast_settled_q(q, N.fix_eq, f)) return f;
    }
    return (float)nn_d_y0(N, T, x, z, xc, zc);
}
/* a value only quantised, from a fixed-point approximation q (units of 2^-59) within eq units of the
 * reference's double value v: true when every real in [q - eq, q + eq] 2^-59 has the target of the two ends
 * (the rounding to float, the product by 10000 and the truncation are each monotone, so the ends settle
 * quantize((float)v)); f is then a float with that target (the lower end's) */
__device__ __forceinline__ bool quant_settled_q(int64_t q, int64_t eq, float &f) {
    const float lo = __ll2float_rn(q - eq) * 0x1.0p-59f, hi = __ll2float_rn(q + eq) * 0x1.0p-59f;
    f = lo;
    return quantize(lo) == quantize(hi);
}
/* a float with the target of a double-branch NormalNoise's value at (x, 0, z), for a noise whose float is
 * only quantised (the Nether's two): the 32-bit screen's when it settles the target, else nn_d_y0_float's
 * (the float itself).  The Overworld's temperature and vegetation are only quantised too, but there the
 * second octave form measured slower: its code pushed the double branch's hot path out of the instruction
 * cache. */
__device__ __forceinline__ float nn_d_y0_qfloat(const MgNoise &N, const MgLattice *__restrict__ T, double x, double z,
                                                double xc, double zc) {
    float f;
    if (N.fix_eq32 >= 0) {
        const int64_t q = nn_q32(N, T, x, z, xc, zc);
        if (q != MG_QFAIL && quant_settled_q(q, N.fix_eq32, f)) return f;
    }
    return nn_d_y0_float(N, T, x, z, xc, zc);
}
/* ridges_folded (|(|r| + c0)| + c1) * c2 of a ridge value (the exact path) */
__device__ __forceinline__ double ridges_folded_d(const MgWorldDesc &W, double r) {
    return (fabs(fabs(r) + W.rf_d[0]) + W.rf_d[1]) * W.rf_d[2];
}
/* the float of ridges_folded from a fixed-point ridge value q (units of 2^-59) within the ridge screen's
 * bound: the constants are multiples of 2^-59 (W.rf_eq >= 0), so the sums are exact and the product rounds
 * down by less than one unit (it runs for sums below 4; others go to the exact path).  ridges_folded of two
 * values within d of each other differ by at most |c2| d, and the reference's three roundings of it (values
 * below 17) by less than |c2| 1e-14 + 1e-13, so W.rf_eq is |c2| (err + 1e-14) + 1e-13 plus one unit. */
__device__ __forceinline__ bool ridges_folded_settled(const MgWorldDesc &W, int64_t q, float &f) {
    int64_t v = (q < 0 ? -q : q) + W.rf_q[0];
    v = (v < 0 ? -v : v) + W.rf_q[1];
    if (v >= (4LL << MG_Q) || v <= -(4LL << MG_Q)) return false;
    const int64_t c = W.rf_q[2], m = mulq_us(c < 0 ? -c : c, v);
    return cast_settled_q(c < 0 ? -m : m, W.rf_eq, f);
}
/* ridge noise and ridges_folded as floats */
__device__ __forceinline__ void ridge_float(const MgWorldDesc &W, const MgLattice *__restrict__ T, double x, double z,
                                            double xc, double zc, float &rvf, float &rff) {
    const MgNoise &N = W.noise[5];
    if (W.rf_eq >= 0) {
        const int64_t q = nn_q<false>(N, T, x, z, xc, zc);
        if (q != MG_QFAIL && cast_settled_q(q, N.fix_eq, rvf) && ridges_folded_settled(W, q, rff))
            return;
    }
    const double rv = nn_d_y0(N, T, x, z, xc, zc);
    rvf = (float)rv;
    rff = (float)ridges_folded_d(W, rv);
}

/* double branch of the Overworld climate after the shift: the climate noises screened at the exact shifted
 * coordinates, the finish (out of line: reached from the per-cell and the per-tile shift forms) */
static __device__ __noinline__ void climate_ow_d_rest(const MgWorldDesc &W, const MgSpline &S, const MgLattice *__restrict__ T,
                                                      double x, double z, double g, int32_t *tg) {
    const double xc = x * MG_SECOND_STACK, zc = z * MG_SECOND_STACK;
    const float tf = nn_d_y0_float(W.noise[1], T, x, z, xc, zc);
    const float hf = nn_d_y0_float(W.noise[2], T, x, z, xc, zc);
    const float cf = nn_d_y0_float(W.noise[3], T, x, z, xc, zc);
    const float ef = nn_d_y0_float(W.noise[4], T, x, z, xc, zc);
    float rvf, rff;
    ridge_float(W, T, x, z, xc, zc, rvf, rff);
    climate_finish_df(W, S, tf, hf, cf, ef, rvf, rff, g, tg);
}
/* Where a batch records the cells whose screened climate left a value to the exact evaluation (MgPending):
 * the record array, its counter and capacity, and the request's world and lattices. */
struct PendSink {
    MgPending *rec;
    unsigned long long *count;
    long long cap;
    int32_t world, state;
};
/* the rare part of climate_ow_d_rest_defer (a value the screen left unsettled), out of line so that the hot
 * path stays compact: the cell recorded in the sink (recorded true), or, the sink full or absent, the unsettled
 * values evaluated exactly in place (fv updated) */
struct F6 {
    float v[6];
};
struct DeferOut {
    F6 f;
    bool recorded;
};
static __device__ __noinline__ DeferOut defer_or_exact(const MgWorldDesc &W, const MgLattice *__restrict__ T, double x,
                                                      double z, double g, uint32_t pend, const PendSink *sink,
                                                      int64_t out, F6 fv) {
    const double xc = x * MG_SECOND_STACK, zc = z * MG_SECOND_STACK;
    const unsigned long long k = sink->cap > 0 ? atomicAdd(sink->count, 1ULL) : ~0ULL;
    if (k < (unsigned long long)sink->cap) {
        MgPending &P = sink->rec[k];
        P.x = x;
        P.z = z;
        P.g = g;
        P.out = out;
        for (int j = 0; j < 4; j++) P.f[j] = fv.v[j];
        P.rv = fv.v[4];
        P.rf = fv.v[5];
        P.world = sink->world;
        P.state = sink->state;
        P.pend = pend;
        return DeferOut{fv, true};
    }
    for (int j = 0; j < 4; j++)
        if (pend & (1u << j)) fv.v[j] = (float)nn_d_y0(W.noise[1 + j], T, x, z, xc, zc);
    if (pend & 16u) {
        const double rv = nn_d_y0(W.noise[5], T, x, z, xc, zc);
        fv.v[4] = (float)rv;
        fv.v[5] = (float)ridges_folded_d(W, rv);
    }
    return DeferOut{fv, false};
}
/* climate_ow_d_rest for a batch: the same values, but a cell with a value the screen does not settle is
 * recorded in the sink (output byte `out`) and false returned, without the exact evaluation; when the sink
 * is full (or absent) the exact evaluation runs here and the targets are returned as climate_ow_d_rest gives
 * them. */
static __device__ __noinline__ bool climate_ow_d_rest_defer(const MgWorldDesc &W, const MgSpline &S,
                                                            const MgLattice *__restrict__ T, double x, double z,
                                                            double g, int32_t *tg, const PendSink *sink, int64_t out) {
    const double xc = x * MG_SECOND_STACK, zc = z * MG_SECOND_STACK;
    float fv[6];
    uint32_t pend = 0;
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const MgNoise &N = W.noise[1 + k];
        const int64_t q = N.fix_eq >= 0 ? nn_q<false>(N, T, x, z, xc, zc) : MG_QFAIL;
        if (q == MG_QFAIL || !cast_settled_q(q, N.fix_eq, fv[k])) pend |= 1u << k;
    }
    {
        const MgNoise &N = W.noise[5];
        const int64_t q = W.rf_eq >= 0 ? nn_q<false>(N, T, x, z, xc, zc) : MG_QFAIL;
        if (q == MG_QFAIL || !cast_settled_q(q, N.fix_eq, fv[4]) || !ridges_folded_settled(W, q, fv[5])) pend |= 16u;
    }
    if (pend) {
        const DeferOut r = defer_or_exact(W, T, x, z, g, pend, sink, out, F6{{fv[0], fv[1], fv[2], fv[3], fv[4], fv[5]}});
        if (r.recorded) return false;
        for (int j = 0; j < 6; j++) fv[j] = r.f.v[j];
    }
    climate_finish_df(W, S, fv[0], fv[1], fv[2], fv[3], fv[4], fv[5], g, tg);
    return true;
}
/* a recorded cell's targets: its settled floats and the exact evaluation of the rest (the values
 * climate_ow_d_rest computes) */
__device__ __forceinline__ void pending_targets(const MgWorldDesc &W, const MgLattice *__restrict__ T, const MgPending &P,
                                                int32_t *tg) {
    const double xc = P.x * MG_SECOND_STACK, zc = P.z * MG_SECOND_STACK;
    float fv[6] = {P.f[0], P.f[1], P.f[2], P.f[3], P.rv, P.rf};
#pragma unroll
    for (int j = 0; j < 4; j++)
        if (P.pend & (1u << j)) fv[j] = (float)nn_d_y0(W.noise[1 + j], T, P.x, P.z, xc, zc);
    if (P.pend & 16u) {
        const double rv = nn_d_y0(W.noise[5], T, P.x, P.z, xc, zc);
        fv[4] = (float)rv;
        fv[5] = (float)ridges_folded_d(W, rv);
    }
    climate_finish_df(W, W.spline, fv[0], fv[1], fv[2], fv[3], fv[4], fv[5], P.g, tg);
}

/* double branch of the Overworld climate, out of line (the kernels reach the climate from two sites each:
 * the cell itself and the tie chain).  The shift noises stay exact in double: their value moves the climate
 * noises' input coordinates, and the kernels' integer pipes (which carry the screened climate noises) are
 * busier than the FP64 pipe, so a fixed-point shift measured slower. */
static __device__ __noinline__ void climate_ow_d(const MgWorldDesc &W, const MgSpline &S, const MgLattice *__restrict__ T,
                                                 double X, double Z, double Xc, double Zc, int by, int32_t *tg) {
    const double sx = nn_d_y0(W.noise[0], T, X, Z, Xc, Zc) * 4.0;
    const double sz = nn_d_z0(W.noise[0], T, Z, X, Zc, Xc) * 4.0;
    climate_ow_d_rest(W, S, T, X + sx, Z + sz, depth_grad_d(W, by), tg);
}

/* Shift noises of a tile, double branch.  Every input of ShiftA (x, 0, z) and ShiftB (z, x, 0) depends on
 * one coordinate: X f + o or Z f + o (first stack), X c f + o or Z c f + o (second stack).  So the cells of a
 * tile column share their X-side splits and smoothsteps, the cells of a row their Z-side ones, and the CTA
 * computes them once per tile into a table (entry (lattice, family, column or row); families: X with the
 * lattice's x offset (ShiftA's x input), X with its y offset (ShiftB's y input), Z with its z offset
 * (ShiftA's z input), Z with its x offset (ShiftB's x input)).  Each cell then runs only the octaves'
 * gradient sums and lerps: the splits and smoothsteps are the per-cell functions' values on the same
 * inputs, so the result is the same to the bit. */
#define SHIFT_MAXLEV 3                        /* levels of the shift noise the table serves (26.x: 3) */
struct ShiftSplit {
    int64_t pk;                               /* fraction in units of 2^-52 | (cell & 255) << 52; -1: not a multiple */
    double u;                                 /* smoothstep of the fraction */
};
template <int TW, int TH>
struct ShiftTable {
    ShiftSplit e[2 * SHIFT_MAXLEV][2 * TW + 2 * TH]; /* per lattice: X+ox, X+oy (TW each), Z+oz, Z+ox (TH each) */
};
/* true when the world's shift noise fits the table */
__device__ __forceinline__ bool shift_table_ok(const MgWorldDesc &W) { return W.noise[0].nlev <= SHIFT_MAXLEV; }
/* the table of the tile whose first cell is (qx0, qz0); all threads of the block take part */
template <int TW, int TH, int NT>
__device__ __forceinline__ void shift_table_fill(const MgNoise &N, const MgLattice *__restrict__ T, int qx0, int qz0,
                                                 ShiftTable<TW, TH> &tab) {
    const int per = 2 * TW + 2 * TH, nl = 2 * N.nlev;
    const MgLattice *A = T + N.base;
    for (int e = threadIdx.x; e < nl * per; e += NT) {
        const int j = e / per, r = e % per; /* r: the entry's place in the lattice's row of the table */
        const int fam = r < 2 * TW ? r / TW : 2 + (r - 2 * TW) / TH;
        const int idx = r < 2 * TW ? r % TW : (r - 2 * TW) % TH;
        const int st = j >= N.nlev, k = j - st * N.nlev;
        const MgLattice *L = A + j;
        double c = fam < 2 ? (double)(qx0 + idx) : (double)(qz0 + idx);
        if (st) c = c * MG_SECOND_STACK;
        const double off = fam == 0 ? L->ox : (fam == 1 ? L->oy : (fam == 2 ? L->oz : L->ox));
        int i;
        double fr;
        int64_t F;
        split_dk(c, N.freq[k], N.fexp[k], off, i, fr, F);
        ShiftSplit &o = tab.e[j][r];
        o.pk = F < 0 ? -1 : (F | ((int64_t)(i & 255) << 52));
        o.u = F < 0 ? 0.0 : fade<double>(fr);
    }
}
struct ShiftPair {
    double a, b; /* ShiftA, ShiftB */
    bool ok;
};
/* both shift noises of the cell in column col and row row from the table (same sums as nn_d); ok false when
 * an entry or a zero coordinate's split is not a multiple of 2^-52 (the per-cell form handles the cell) */
template <int TW, int TH>
static __device__ __noinline__ ShiftPair shift_from_table(const MgNoise &N, const MgLattice *__restrict__ T,
                                                          const ShiftTable<TW, TH> &tab, int col, int row) {
    const int64_t M52 = (1LL << 52) - 1;
    double sa[2] = {0.0, 0.0}, sb[2] = {0.0, 0.0};
    const MgLattice *A = T + N.base;
    /* one octave per step (ShiftA and ShiftB of each level and stack in turn; each sum keeps its order): one
     * copy of the octave code, where two per step measured slower, the hot code no longer fitting the
     * instruction cache */
#pragma unroll 1
    for (int e = 0; e < 4 * N.nlev; e++) {
        const int q = e >> 1, isb = e & 1, k = q >> 1, st = q & 1, j = st * N.nlev + k;
        const MgLattice *L = A + j;
        const ShiftSplit ex = tab.e[j][col], ey = tab.e[j][TW + col], ez = tab.e[j][2 * TW + row],
                         ew = tab.e[j][2 * TW + TH + row];
        if ((ex.pk | ey.pk | ez.pk | ew.pk | L->Fy | L->Fz) < 0) return ShiftPair{0.0, 0.0, false};
        const PlainPerm p{L->p};
        const ShiftSplit sx = isb ? ew : ex, sz = isb ? ey : ez;
        const int ix = (int)(sx.pk >> 52), iy = isb ? (int)(sz.pk >> 52) : L->iy;
        const int64_t FX = sx.pk & M52, FY = isb ? (sz.pk & M52) : L->Fy;
        const double u = sx.u, v = isb ? sz.u : L->uyd;
        const int iz = isb ? L->iz : (int)(sz.pk >> 52);
        const int64_t FZ = isb ? L->Fz : (sz.pk & M52);
        const double w = isb ? L->uzd : sz.u;
        const double o = octave_dfix_u(p, ix, FX, u, iy, FY, v, iz, FZ, w);
        const double t = N.amp_d[k] * o * N.vf_d[k];
        if (isb) { if (st) sb[1] += t; else sb[0] += t; }
        else { if (st) sa[1] += t; else sa[0] += t; }
    }
    return ShiftPair{(sa[0] + sa[1]) * N.vfac, (sb[0] + sb[1]) * N.vfac, true};
}
/* the double branch's Overworld climate of a tile cell, the shifts from the tile's table; g the tile's depth
 * gradient, depth_grad_d(W, 4 qy) */
template <int TW, int TH>
__device__ __forceinline__ void climate_ow_d_tab(const MgWorldDesc &W, const MgSpline &S, const MgLattice *__restrict__ T,
                                                 const ShiftTable<TW, TH> &tab, int col, int row, int qx, int qy, int qz,
                                                 double g, int32_t *tg) {
    const ShiftPair sp = shift_from_table(W.noise[0], T, tab, col, row);
    const double X = (double)qx, Z = (double)qz;
    if (!sp.ok) {
        climate_ow_d(W, S, T, X, Z, X * MG_SECOND_STACK, Z * MG_SECOND_STACK, qy * 4, tg);
        return;
    }
    climate_ow_d_rest(W, S, T, X + sp.a * 4.0, Z + sp.b * 4.0, g, tg);
}

/* The float branch's shift noises of a tile from a table, as the double branch's: the entries are the float
 * splits (cell, fraction) and the fraction's smoothstep that oct_f computes per cell, on the same inputs (the
 * same families of X- and Z-side coordinates), so each cell's octaves run on the same values and give the same
 * bits; the sums keep nn_f's order. */
struct ShiftSplitF {
    int32_t i;  /* cell */
    float f, u; /* fraction, its smoothstep */
};
template <int TW, int TH>
struct ShiftTableF {
    ShiftSplitF e[2 * SHIFT_MAXLEV][2 * TW + 2 * TH]; /* per lattice: X+ox, X+oy (TW each), Z+oz, Z+ox (TH each) */
};
template <int TW, int TH, int NT>
__device__ __forceinline__ void shift_table_fill_f(const MgNoise &N, const MgLattice *__restrict__ T, int qx0, int qz0,
                                                   ShiftTableF<TW, TH> &tab) {
    const int per = 2 * TW + 2 * TH, nl = 2 * N.nlev;
    const MgLattice *A = T + N.base;
    for (int e = threadIdx.x; e < nl * per; e += NT) {
        const int j = e / per, r = e % per;
        const int fam = r < 2 * TW ? r / TW : 2 + (r - 2 * TW) / TH;
        const int idx = r < 2 * TW ? r % TW : (r - 2 * TW) % TH;
        const int st = j >= N.nlev, k = j - st * N.nlev;
        const MgLattice *L = A + j;
        double c = fam < 2 ? (double)(qx0 + idx) : (double)(qz0 + idx);
        if (st) c = c * MG_SECOND_STACK;
        const double off = fam == 0 ? L->ox : (fam == 1 ? L->oy : (fam == 2 ? L->oz : L->ox));
        int i;
        float fr;
        split_fk(c, N.freq[k], N.fexp[k], off, i, fr);
        ShiftSplitF &o = tab.e[j][r];
        o.i = i;
        o.f = fr;
        o.u = fade<float>(fr);
    }
}
/* ShiftA and ShiftB of the cell in column col and row row (nn_f's values: level by level, first stack then
 * second, each sum in its own order), one octave per loop step */
template <int TW, int TH>
static __device__ __noinline__ float2 shift_from_table_f(const MgNoise &N, const MgLattice *__restrict__ T,
                                                         const ShiftTableF<TW, TH> &tab, int col, int row) {
    float sa = 0.0f, sb = 0.0f;
    const MgLattice *A = T + N.base;
#pragma unroll 1
    for (int e = 0; e < 4 * N.nlev; e++) {
        const int q = e >> 1, isb = e & 1, k = q >> 1, st = q & 1, j = st * N.nlev + k;
        const MgLattice *L = A + j;
        /* ShiftA (x, 0, z): x input X + ox, z input Z + oz, y from the header; ShiftB (z, x, 0): x input Z + ox,
         * y input X + oy, z from the header */
        const ShiftSplitF ex = isb ? tab.e[j][2 * TW + TH + row] : tab.e[j][col];
        const ShiftSplitF eo = isb ? tab.e[j][TW + col] : tab.e[j][2 * TW + row];
        const int iy = isb ? eo.i : L->iy, iz = isb ? L->iz : eo.i;
        const float fy = isb ? eo.f : L->z0.f.fy, fz = isb ? L->z0.f.fz : eo.f;
        const float v = isb ? eo.u : L->z0.f.uy, w = isb ? L->z0.f.uz : eo.u;
        const float o = octave_q<float>(PlainPerm{L->p}, ex.i, ex.f, iy, fy, fy - 1.0f, v, iz, fz, fz - 1.0f, w);
        const float t = N.amp_f[k] * o;
        if (isb) sb += t;
        else sa += t;
    }
    return make_float2(sa, sb);
}
/* the float branch's Overworld climate of a tile cell, the shifts from the tile's table (climate_ow<true>'s
 * values) */
template <int TW, int TH>
__device__ __forceinline__ void climate_ow_f_tab(const MgWorldDesc &W, const MgSpline &S, const MgLattice *__restrict__ T,
                                                 const ShiftTableF<TW, TH> &tab, int col, int row, int qx, int qy, int qz,
                                                 int32_t tg[6]) {
    const double X = (double)qx, Z = (double)qz;
    const float2 sh = shift_from_table_f(W.noise[0], T, tab, col, row);
    const float sx = sh.x * 4.0f, sz = sh.y * 4.0f;
    const double x = X + (double)sx, z = Z + (double)sz;
    const double xc = x * MG_SECOND_STACK, zc = z * MG_SECOND_STACK;
    const float tv = nn_f_y0(W.noise[1], T, x, z, xc, zc);
    const float hv = nn_f_y0(W.noise[2], T, x, z, xc, zc);
    const float cv = nn_f_y0(W.noise[3], T, x, z, xc, zc);
    const float ev = nn_f_y0(W.noise[4], T, x, z, xc, zc);
    const float rv = nn_f_y0(W.noise[5], T, x, z, xc, zc);
    climate_finish_f(W, S, tv, hv, cv, ev, rv, qy * 4, tg);
}

/* climate_ow_d_tab with the deferral of climate_ow_d_rest_defer */
template <int TW, int TH>
__device__ __forceinline__ bool climate_ow_d_tab_defer(const MgWorldDesc &W, const MgSpline &S,
                                                       const MgLattice *__restrict__ T, const ShiftTable<TW, TH> &tab,
                                                       int col, int row, int qx, int qy, int qz, double g, int32_t *tg,
                                                       const PendSink *sink, int64_t out) {
    const ShiftPair sp = shift_from_table(W.noise[0], T, tab, col, row);
    const double X = (double)qx, Z = (double)qz;
    if (!sp.ok) {
        climate_ow_d(W, S, T, X, Z, X * MG_SECOND_STACK, Z * MG_SECOND_STACK, qy * 4, tg);
        return true;
    }
    return climate_ow_d_rest_defer(W, S, T, X + sp.a * 4.0, Z + sp.b * 4.0, g, tg, sink, out);
}

/* Overworld climate of quart cell (qx, qy, qz) -> 6 quantised targets (engine/mc_climate.h:113-170). */
template <bool FM>
__device__ __forceinline__ void climate_ow(const MgWorldDesc &W, const MgSpline &S, const MgLattice *__restrict__ T,
                                           int qx, int qy, int qz, int32_t tg[6]) {
    const double X = (double)qx, Z = (double)qz; /* blockX * 0.25 with blockX = 4 qx */
    const double Xc = X * MG_SECOND_STACK, Zc = Z * MG_SECOND_STACK;
    const int by = qy * 4;
    if (FM) {
        float sx = nn_f_y0(W.noise[0], T, X, Z, Xc, Zc) * 4.0f; /* ShiftA (x, 0, z) */
        float sz = nn_f_z0(W.noise[0], T, Z, X, Zc, Xc) * 4.0f; /* ShiftB (z, x, 0) */
        double x = X + (double)sx, z = Z + (double)sz;
        double xc = x * MG_SECOND_STACK, zc = z * MG_SECOND_STACK;
        float tv = nn_f_y0(W.noise[1], T, x, z, xc, zc);
        float hv = nn_f_y0(W.noise[2], T, x, z, xc, zc);
        float cv = nn_f_y0(W.noise[3], T, x, z, xc, zc);
        float ev = nn_f_y0(W.noise[4], T, x, z, xc, zc);
        float rv = nn_f_y0(W.noise[5], T, x, z, xc, zc);
        climate_finish_f(W, S, tv, hv, cv, ev, rv, by, tg);
    } else {
        climate_ow_d(W, S, T, X, Z, Xc, Zc, by, tg);
    }
}
/* Nether: temperature and vegetation at (x/4, 0, z/4) (engine/cuda/mcg_host.c:63-74) */
template <bool FM>
__device__ __forceinline__ void climate_nether(const MgWorldDesc &W, const MgLattice *__restrict__ T, int qx, int qz,
                                               int32_t tg[6]) {
    const double X = (double)qx, Z = (double)qz;
    const double Xc = X * MG_SECOND_STACK, Zc = Z * MG_SECOND_STACK;
    float t, h;
    if (FM) {
        t = nn_f_legacy_y0(W.nether[0], T, X, Z, Xc, Zc);
        h = nn_f_legacy_y0(W.nether[1], T, X, Z, Xc, Zc);
    } else {
        t = nn_d_y0_qfloat(W.nether[0], T, X, Z, Xc, Zc);
        h = nn_d_y0_qfloat(W.nether[1], T, X, Z, Xc, Zc);
    }
    tg[0] = quantize(t);
    tg[1] = quantize(h);
    tg[2] = tg[3] = tg[4] = tg[5] = 0;
}
template <bool FM, int DIM>
__device__ __forceinline__ void cell_target(const MgWorldDesc &W, const MgSpline &S, const MgLattice *__restrict__ T,
                                            int qx, int qy, int qz, int32_t tg[6]) {
    if (DIM == MG_OVERWORLD) climate_ow<FM>(W, S, T, qx, qy, qz, tg);
    else climate_nether<FM>(W, T, qx, qz, tg);
}

/* ============================================================================ End islands (engine/mc_end.h) */
__device__ __forceinline__ double simplex2(const uint8_t *__restrict__ p, double xin, double yin, double F2, double G2) {
    double s = (xin + yin) * F2;
    int i = ifloor(xin + s), j = ifloor(yin + s);
    double t = (double)(i + j) * G2;
    double x0 = xin - ((double)i - t), y0 = yin - ((double)j - t);
    int i1 = x0 > y0 ? 1 : 0, j1 = 1 - i1;
    double x1 = x0 - (double)i1 + G2, y1 = y0 - (double)j1 + G2;
    double x2 = x0 - 1.0 + 2.0 * G2, y2 = y0 - 1.0 + 2.0 * G2;
    int ii = i & 255, jj = j & 255;
    int g0 = p[(ii + p[jj]) & 255] % 12;
    int g1 = p[(ii + i1 + p[(jj + j1) & 255]) & 255] % 12;
    int g2 = p[(ii + 1 + p[(jj + 1) & 255]) & 255] % 12;
    double n = 0.0, acc[3];
    const double xs[3] = {x0, x1, x2}, ys[3] = {y0, y1, y2};
    const int gs[3] = {g0, g1, g2};
#pragma unroll
    for (int c = 0; c < 3; c++) {
        double tt = 0.5 - xs[c] * xs[c] - ys[c] * ys[c] - 0.0 * 0.0;
        if (tt < 0.0) acc[c] = 0.0;
        else {
            tt *= tt;
            acc[c] = tt * tt * gdot<double>(gs[c], xs[c], ys[c], 0.0);
        }
    }
    n = acc[0] + acc[1] + acc[2];
    return 70.0 * n;
}
/* End island test, screened: the reference decides an island cell by nv < -0.9f (double branch, the float
 * constant widened) or (float)nv < -0.9f (float branch), nv = simplex2 in double (about 60 FP64-pipe
 * operations).  Here the skew, the cell (i, j), the corner choice and the first corner's offsets x0, y0 are
 * the reference's double arithmetic (exact same values), and the three corner terms are evaluated in float
 * from those offsets: |float value - nv| <= END_ISLAND_E (a forward error bound: offsets within 5 u of the
 * double ones, u = 2^-24; tt = 0.5 - x^2 - y^2 within 32 u; tt^4 within 18 u; the gradient dot within 12 u;
 * each term tt^4 * dot within 26 u for |x|, |y| < 0.71 (tt > 0); three terms and their sums within 78 u; times
 * 70: 5,500 u = 3.3e-4 plus the reference's own double roundings, taken as 5e-4).  A value farther than that
 * from the threshold settles the test (with one more float ulp for the float branch's rounding); the rest
 * (a few in 10^4) take the exact double evaluation.  mcgen_gb300_check_end checks the bound and the decisions
 * on the device. */
#define END_ISLAND_E 5e-4f
__device__ __forceinline__ bool end_island(const uint8_t *__restrict__ p, double xin, double yin, double F2, double G2,
                                           bool fm) {
    const double s = (xin + yin) * F2;
    const int i = ifloor(xin + s), j = ifloor(yin + s);
    const double t = (double)(i + j) * G2;
    const double x0 = xin - ((double)i - t), y0 = yin - ((double)j - t);
    const int i1 = x0 > y0 ? 1 : 0, j1 = 1 - i1;
    const float g2 = (float)G2, xf = (float)x0, yf = (float)y0;
    const float xs[3] = {xf, xf - (float)i1 + g2, xf - 1.0f + 2.0f * g2};
    const float ys[3] = {yf, yf - (float)j1 + g2, yf - 1.0f + 2.0f * g2};
    const int ii = i & 255, jj = j & 255;
    const int gs[3] = {p[(ii + p[jj]) & 255] % 12, p[(ii + i1 + p[(jj + j1) & 255]) & 255] % 12,
                       p[(ii + 1 + p[(jj + 1) & 255]) & 255] % 12};
    float n = 0.0f;
#pragma unroll
    for (int c = 0; c < 3; c++) {
        float tt = 0.5f - xs[c] * xs[c] - ys[c] * ys[c];
        if (tt > 0.0f) {
            tt *= tt;
            n += tt * tt * gdot<float>(gs[c], xs[c], ys[c], 0.0f);
        }
    }
    n *= 70.0f;
    if (n < -0.9f - (END_ISLAND_E + 1e-4f)) return true; /* nv < -0.9f - ulp: an island in both branches */
    if (n >= -0.9f + (END_ISLAND_E + 1e-4f)) return false; /* nv > -0.9f: none */
    const double nv = simplex2(p, xin, yin, F2, G2);
    return fm ? ((float)nv < -0.9f) : (nv < (double)-0.9f);
}
__device__ __forceinline__ float clampf(float v, float lo, float hi) { return v < lo ? lo : (v < hi ? v : hi); }
/* EndIslandDensityFunction.getHeightValue at (sx, sz) = (block / 8); rad: half-width of the island window in
 * chunk cells (12 in the game; the seed search may narrow it, engine/cuda/mc_gpu.cuh:600-626, 640-652) */
inline __device__ float end_height(const uint8_t *__restrict__ p, bool fm, int sx, int sz, double F2, double G2,
                                   int rad = 12) {
    int cx = sx / 2, cz = sz / 2, ox = sx % 2, oz = sz % 2;
    float best;
    if (!fm) {
        int32_t sq = (int32_t)((uint32_t)sx * (uint32_t)sx + (uint32_t)sz * (uint32_t)sz); /* Java int overflow */
        float len = (float)sqrt((double)(float)sq);
        best = clampf(100.0f - len * 8.0f, -100.0f, 80.0f);
    } else best = -100.0f;
    for (int dx = -rad; dx <= rad; dx++)
        for (int dz = -rad; dz <= rad; dz++) {
            long long tx = (long long)cx + dx, tz = (long long)cz + dz;
            if (tx * tx + tz * tz <= 4096LL) continue;
            if (!end_island(p, (double)tx, (double)tz, F2, G2, fm)) continue;
            float size = fmodf(fabsf((float)tx) * 3439.0f + fabsf((float)tz) * 147.0f, 13.0f) + 9.0f;
            float xd = (float)(ox - dx * 2), zd = (float)(oz - dz * 2);
            float h = clampf(100.0f - (float)sqrt((double)(xd * xd + zd * zd)) * size, -100.0f, 80.0f);
            best = best > h ? best : h;
        }
    return best;
}
/* TheEndBiomeSource class of chunk (cx, cz): 0 the_end, 1 highlands, 2 midlands, 3 small islands, 4 barrens */
inline __device__ int end_chunk_class(const uint8_t *__restrict__ p, bool fm, int cx, int cz, double F2, double G2,
                                      int rad = 12) {
    if ((long long)cx * cx + (long long)cz * cz <= 4096LL) return 0;
    int bx = (cx * 2 + 1) * 8, bz = (cz * 2 + 1) * 8;
    float h = end_height(p, fm, bx / 8, bz / 8, F2, G2, rad);
    double e;
    if (!fm) e = ((double)h - 8.0) / 128.0;
    else {
        float dx = (float)(0 - bx), dz = (float)(0 - bz);
        float len = (float)sqrt((double)(dx * dx + 0.0f * 0.0f + dz * dz));
        float c = (clampf(100.0f - len, -100.0f, 80.0f) - 8.0f) * 0.0078125f;
        float o = (h - 8.0f) / 128.0f;
        e = (double)(c > o ? c : o);
    }
    if (e > 0.25) return 1;
    if (e >= -0.0625) return 2;
    return e < -0.21875 ? 3 : 4;
}

/* ---------------------------------------------------------------------------- BiomeManager zoom
 * (libmcgen/src/region.c:61-85) */
__device__ __forceinline__ int64_t zoom_step(int64_t r, int64_t c) {
    uint64_t v = (uint64_t)r;
    v *= v * 6364136223846793005ULL + 1442695040888963407ULL;
    return (int64_t)(v + (uint64_t)c);
}
/* Math.floorMod(r >> 24, 1024) / 1024.0: the ten bits above bit 23; the division by 2^10 is exact as a scaling */
__device__ __forceinline__ int zoom_bits(int64_t r) { return (int)((r >> 24) & 1023); }
__device__ __forceinline__ double zoom_jitter(int m) { return ((double)m * 0x1.0p-10 - 0.5) * 0.9; }
/* the three jitter draws of candidate cell (x, y, z), ten bits each (x in bits 0-9, y 10-19, z 20-29) */
__device__ __forceinline__ uint32_t zoom_draws(int64_t seed, int x, int y, int z) {
    int64_t r = seed;
    r = zoom_step(r, x); r = zoom_step(r, y); r = zoom_step(r, z);
    r = zoom_step(r, x); r = zoom_step(r, y); r = zoom_step(r, z);
    uint32_t m = (uint32_t)zoom_bits(r);
    r = zoom_step(r, seed);
    m |= (uint32_t)zoom_bits(r) << 10;
    r = zoom_step(r, seed);
    return m | (uint32_t)zoom_bits(r) << 20;
}
/* the fiddled distance in double, in the reference's order (z, y, x terms) */
__device__ __forceinline__ double zoom_dist_d(uint32_t m, double dx, double dy, double dz) {
    const double jx = zoom_jitter((int)(m & 1023)), jy = zoom_jitter((int)((m >> 10) & 1023)),
                 jz = zoom_jitter((int)(m >> 20));
    return (dz + jz) * (dz + jz) + (dy + jy) * (dy + jy) + (dx + jx) * (dx + jx);
}
/* The same in single precision, as a screen.  Against the double value it differs by at most 1.23e-6: each
 * of the three squared terms by at most 2.48e-7 (the maximum over all 8 x 1024 (offset, draw) pairs, the
 * draw's jitter taken as (m - 512) * fl32(0.9 / 1024)), and the two single-precision additions of terms below
 * 6.31 by half an ulp (2^-22) each.  So a candidate whose screened distance exceeds the smallest screened one
 * by more than ZOOM_MARGIN (four times twice that bound) cannot be the double-precision minimum. */
#define ZOOM_MARGIN 1e-5f
__device__ __forceinline__ float zoom_dist_f(uint32_t m, int qx, int qy, int qz) {
    const float c = 0.9f / 1024.0f;
    const float ux = (float)qx * 0.25f + (float)((int)(m & 1023) - 512) * c;
    const float uy = (float)qy * 0.25f + (float)((int)((m >> 10) & 1023) - 512) * c;
    const float uz = (float)qz * 0.25f + (float)((int)(m >> 20) - 512) * c;
    return uz * uz + uy * uy + ux * ux;
}
/* BiomeManager.getBiome's choice among the 8 quart cells around block (x, y, z): the first candidate (in the
 * order x, y, z bit = 0 first) with the smallest double-precision fiddled distance.  The distances are
 * screened in single precision; only when a second candidate lies within ZOOM_MARGIN of the smallest are the
 * close candidates' distances taken in double precision (in candidate order, strict comparison), which
 * gives the same choice as the double-precision comparison of all 8. */
__device__ __forceinline__ int zoom_pick(int64_t zseed, int px, int py, int pz, int fx, int fy, int fz, int &close) {
    uint32_t mm[8];
    float df[8];
    float bf = __int_as_float(0x7F800000);
#pragma unroll
    for (int i = 0; i < 8; i++) {
        const int ox = (i >> 2) & 1, oy = (i >> 1) & 1, oz = i & 1;
        mm[i] = zoom_draws(zseed, px + ox, py + oy, pz + oz);
        df[i] = zoom_dist_f(mm[i], fx - 4 * ox, fy - 4 * oy, fz - 4 * oz);
        bf = fminf(bf, df[i]);
    }
    const float lim = bf + ZOOM_MARGIN;
    int best = -1;
    close = 0;
#pragma unroll
    for (int i = 0; i < 8; i++)
        if (df[i] <= lim) { close++; if (best < 0) best = i; }
    if (close > 1) {
        double bd = __longlong_as_double(0x7FF0000000000000LL);
#pragma unroll
        for (int i = 0; i < 8; i++) {
            if (df[i] > lim) continue;
            const int ox = (i >> 2) & 1, oy = (i >> 1) & 1, oz = i & 1;
            const double d = zoom_dist_d(mm[i], fx * 0.25 - ox, fy * 0.25 - oy, fz * 0.25 - oz);
            if (bd > d) { best = i; bd = d; }
        }
    }
    return best;
}
__device__ __forceinline__ void zoom_cell(int64_t zseed, int x, int y, int z, int &cx, int &cy, int &cz) {
    const int ax = x - 2, ay = y - 2, az = z - 2;
    const int px = ax >> 2, py = ay >> 2, pz = az >> 2;
    int close;
    const int best = zoom_pick(zseed, px, py, pz, ax & 3, ay & 3, az & 3, close);
    cx = px + ((best >> 2) & 1);
    cy = py + ((best >> 1) & 1);
    cz = pz + (best & 1);
}
/* The chain of cell_chunk, given the cell's own target tg0 and search (leaf0, the first leaf at the minimum
 * distance d0, and whether another leaf ties it): when the cell is tied, walk back to the first untied cell of
 * the chunk's fill order and replay the chain forward, the cell's own step from tg0, leaf0 and d0 (a tied
 * lane pays one climate evaluation per cell walked back, not two; its warp waits for it). */
template <bool FM, int DIM>
__device__ int cell_chunk_chain(const MgWorldDesc &W, const MgSpline &S, const MgLattice *__restrict__ T,
                                const MgTreeNode *__restrict__ tree, int qx, int qy, int qz, const int32_t *tg0,
                                int leaf0, uint64_t d0, bool tied) {
    const int qmin = W.min_y >> 2, qh = W.height >> 2;
    qy = qy < qmin ? qmin : (qy > qmin + qh - 1 ? qmin + qh - 1 : qy);
    const int bx = qx & ~3, bz = qz & ~3, ly = qy - qmin;
    const int idx0 = (ly >> 2) * 64 + (qx & 3) * 16 + (ly & 3) * 4 + (qz & 3);
    if (idx0 == 0 || !tied) return tree[leaf0].biome;
    int32_t tg[6];
    uint64_t d;
    int idx = idx0 - 1, leaf;
    for (;;) {
        int sec = idx >> 6, r = idx & 63;
        cell_target<FM, DIM>(W, S, T, bx + (r >> 4), qmin + sec * 4 + ((r >> 2) & 3), bz + (r & 3), tg);
        leaf = tree_search_tie(tree, tg, d, tied);
        if (idx == 0 || !tied) break;
        idx--;
    }
    for (int k = idx + 1; k < idx0; k++) { /* replay the chain forward */
        int sec = k >> 6, r = k & 63;
        cell_target<FM, DIM>(W, S, T, bx + (r >> 4), qmin + sec * 4 + ((r >> 2) & 3), bz + (r & 3), tg);
        int l0 = tree_search(tree, tg, -1, d);
        if (node_dist(tree[leaf], tg) != d) leaf = l0;
    }
    if (node_dist(tree[leaf], tg0) != d0) leaf = leaf0; /* the cell's own step */
    return tree[leaf].biome;
}
/* cell_chunk for the 32 neighbouring cells of a warp (all lanes call it, inactive lanes get -1): the cell's
 * own search is the warp-shared walk; the chain (rare) runs per lane. */
template <bool FM, int DIM>
__device__ __forceinline__ int cell_chunk_warp(const MgWorldDesc &W, const MgSpline &S, const MgLattice *__restrict__ T,
                                               const MgTreeNode *__restrict__ tree, int qx, int qy, int qz, bool active,
                                               WarpTreeScratch &ws) {
    const int qmin = W.min_y >> 2, qh = W.height >> 2;
    const int cy = qy < qmin ? qmin : (qy > qmin + qh - 1 ? qmin + qh - 1 : qy);
    int32_t tg[6] = {0, 0, 0, 0, 0, 0};
    if (active) cell_target<FM, DIM>(W, S, T, qx, cy, qz, tg);
    uint64_t d = 0;
    bool tied = false;
    const int leaf = tree_search_tie_warp(tree, tg, active, ws, d, tied);
    if (!active) return -1;
    return cell_chunk_chain<FM, DIM>(W, S, T, tree, qx, qy, qz, tg, leaf, d, tied);
}
/* world_biome_cell (libmcgen/src/biome.c:87-114): y clamped into the dimension; a tied cell walks back along
 * LevelChunkSection.fillBiomesFromNoise order (sections bottom-up, then x, y, z) to an untied cell or the
 * column's first cell, then replays the candidate chain forward.  The walk is bounded by the column.  Out of
 * line: the batch kernel reaches it only for requests under this rule, and inlined its code and registers
 * weighed on the other paths' hot code (spills and the instruction cache). */
template <bool FM, int DIM>
__device__ __noinline__ int cell_chunk(const MgWorldDesc &W, const MgSpline &S, const MgLattice *__restrict__ T,
                                       const MgTreeNode *__restrict__ tree, int qx, int qy, int qz) {
    const int qmin = W.min_y >> 2, qh = W.height >> 2;
    const int cy = qy < qmin ? qmin : (qy > qmin + qh - 1 ? qmin + qh - 1 : qy);
    int32_t tg[6];
    cell_target<FM, DIM>(W, S, T, qx, cy, qz, tg);
    uint64_t d;
    bool tied;
    const int leaf = tree_search_tie(tree, tg, d, tied);
    return cell_chunk_chain<FM, DIM>(W, S, T, tree, qx, qy, qz, tg, leaf, d, tied);
}

}  // namespace mg
#endif
