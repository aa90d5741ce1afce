/* device.cuh -- sm_103a device functions of the biome path.
 *
 * Compiled with --fmad=false and IEEE division/square root: every float/double operation below is
 * rounded separately, in the reference's order, so results are bit-identical to the reference engine
 * (engine/mc_noise.h, mc_climate.h, mc_biomes.h, mc_end.h) and libmcgen's biome map
 * (libmcgen/src/region.c, biome.c).
 */
#ifndef MG_DEVICE_CUH
#define MG_DEVICE_CUH
#include <stdint.h>

#include "mg_types.h"

#define MG_SECOND_STACK 1.0181268882175227 /* NormalNoise second-stack input factor */

namespace mgd {

/* ------------------------------------------------------------------ RNG (engine/mc_rng.h) */
struct Xo { uint64_t lo, hi; };
__device__ __forceinline__ uint64_t rotl64(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
__device__ __forceinline__ uint64_t stafford13(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}
__device__ __forceinline__ Xo xo_make(uint64_t lo, uint64_t hi) {
    Xo r;
    if ((lo | hi) == 0) { lo = 0x9E3779B97F4A7C15ULL; hi = 0x6A09E667F3BCC909ULL; }
    r.lo = lo;
    r.hi = hi;
    return r;
}
/* XoroshiroRandomSource(long): upgradeSeedTo128bit */
__device__ __forceinline__ Xo xo_from_seed(int64_t seed) {
    uint64_t a = (uint64_t)seed ^ 0x6A09E667F3BCC909ULL;
    return xo_make(stafford13(a), stafford13(a + 0x9E3779B97F4A7C15ULL));
}
__device__ __forceinline__ uint64_t xo_next(Xo &r) {
    uint64_t s0 = r.lo, s1 = r.hi;
    uint64_t out = rotl64(s0 + s1, 17) + s0;
    s1 ^= s0;
    r.lo = rotl64(s0, 49) ^ s1 ^ (s1 << 21);
    r.hi = rotl64(s1, 28);
    return out;
}
/* nextInt(bound), Lemire multiply with rejection (XoroshiroRandomSource.nextInt) */
__device__ __forceinline__ int xo_int(Xo &r, uint32_t bound) {
    uint64_t m = (uint64_t)(uint32_t)xo_next(r) * bound;
    if ((uint32_t)m < bound) {
        uint32_t thresh = (0u - bound) % bound;
        while ((uint32_t)m < thresh) m = (uint64_t)(uint32_t)xo_next(r) * bound;
    }
    return (int)(m >> 32);
}
__device__ __forceinline__ double xo_double(Xo &r) { return (double)(xo_next(r) >> 11) * 0x1.0p-53; }

/* java.util.Random LCG */
#define MG_LCG_MUL 0x5DEECE66DULL
#define MG_LCG_MASK 0xFFFFFFFFFFFFULL
__device__ __forceinline__ uint64_t lcg_init(int64_t seed) { return ((uint64_t)seed ^ MG_LCG_MUL) & MG_LCG_MASK; }
__device__ __forceinline__ int32_t lcg_bits(uint64_t &s, int bits) {
    s = (s * MG_LCG_MUL + 0xBULL) & MG_LCG_MASK;
    return (int32_t)(uint32_t)(s >> (48 - bits));
}
/* u % d for u < 2^31 and 2 <= d <= 256 by a multiply-high: with l = ceil(log2 d) and M = ceil(2^(31+l) / d)
 * (< 2^32), floor(u / d) = umulhi(u, M) >> (l - 1) exactly, since M d - 2^(31+l) < d <= 2^l and u < 2^31
 * (Granlund-Montgomery).  The table is indexed by d; in the shuffles every lane of a warp uses the same d. */
struct DivMagic {
    uint32_t m[257];
    uint8_t sh[257];
};
constexpr DivMagic make_div_magic() {
    DivMagic t{};
    for (int d = 2; d <= 256; d++) {
        int l = 0;
        while ((1 << l) < d) l++;
        t.m[d] = (uint32_t)(((1ULL << (31 + l)) + (uint64_t)d - 1) / (uint64_t)d);
        t.sh[d] = (uint8_t)(l - 1);
    }
    return t;
}
static __constant__ DivMagic kDivMagic = make_div_magic();
__device__ __forceinline__ int32_t mod_small(int32_t u, int32_t d) {
    const uint32_t q = __umulhi((uint32_t)u, kDivMagic.m[d]) >> kDivMagic.sh[d];
    return u - (int32_t)q * d;
}
/* java.util.Random.nextInt(bound) for 1 <= bound <= 256 (the permutation shuffles) */
__device__ __forceinline__ int lcg_int(uint64_t &s, int32_t bound) {
    if ((bound & -bound) == bound) return (int)(((int64_t)bound * (int64_t)lcg_bits(s, 31)) >> 31);
    for (;;) {
        int32_t b = lcg_bits(s, 31), v = mod_small(b, bound);
        if ((int32_t)((uint32_t)b - (uint32_t)v + (uint32_t)(bound - 1)) >= 0) return v;
    }
}
__device__ __forceinline__ double lcg_double(uint64_t &s) {
    int64_t hi = lcg_bits(s, 26), lo = lcg_bits(s, 27);
    return (double)((hi << 27) + lo) * 0x1.0p-53;
}
/* s' = A^n s + C_n (mod 2^48): the state after n calls, for a constant step count */
__device__ __forceinline__ uint64_t lcg_jump(uint64_t s, uint32_t n) {
    uint64_t mul = 1, add = 0, cm = MG_LCG_MUL, ca = 0xB;
    while (n) {
        if (n & 1) { mul = (mul * cm) & MG_LCG_MASK; add = (add * cm + ca) & MG_LCG_MASK; }
        ca = ((cm + 1) * ca) & MG_LCG_MASK;
        cm = (cm * cm) & MG_LCG_MASK;
        n >>= 1;
    }
    return (s * mul + add) & MG_LCG_MASK;
}

/* ------------------------------------------------------------------ Java floor */
/* Mth.floor for |v| < 2^31 (cvt.rmi) */
__device__ __forceinline__ int ifloor(double v) { return __double2int_rd(v); }
__device__ __forceinline__ int64_t lfloor(double v) { return __double2ll_rd(v); }

/* Double branch, screened: the octave in 59-bit fixed point (values times 2^59 in int64, |value| < 16),
 * an approximation of the exact real value of the reference's formula.  Products truncate (error below
 * 2^-59 each); sums and the exact-integer gradient sums are exact.  The reference's own double rounding
 * differs from the exact value by far more (the bound used by the screen, MgNoise::fix_err), so the
 * approximation decides the reference's float result except near a float rounding boundary. */
#define MG_Q 59
/* a * b * 2^-59 rounded toward minus infinity, for non-negative operands (the unsigned high product: a
 * signed one costs two sign corrections more) */
__device__ __forceinline__ int64_t mulq_u(int64_t a, int64_t b) {
    const uint64_t hi = __umul64hi((uint64_t)a, (uint64_t)b), lo = (uint64_t)a * (uint64_t)b;
    return (int64_t)((hi << (64 - MG_Q)) | (lo >> MG_Q));
}
/* smoothstep t^3 (6 t^2 - 15 t + 10) of 0 <= t < 1: three products of non-negative values (t^2, t^3, and
 * t^3 p with p in [1, 10]); 6 t^2 and 15 t are shifts and adds */
__device__ __forceinline__ int64_t fadeq(int64_t t) {
    const int64_t t2 = mulq_u(t, t);
    const int64_t p = (t2 << 2) + (t2 << 1) - ((t << 4) - t) + (10LL << MG_Q);
    return mulq_u(mulq_u(t2, t), p);
}

/* ------------------------------------------------------------------ lattice header */
template <typename T>
__device__ __forceinline__ T fade_h(T t) { return t * t * t * (t * (t * (T)6 - (T)15) + (T)10); }
/* d (0 <= d < 1) as a multiple of 2^-52, or -1 when it is not one */
__device__ __forceinline__ int64_t fixed52(double d) {
    const uint64_t b = (uint64_t)__double_as_longlong(d);
    if ((b << 1) == 0) return 0;
    const int e = (int)((b >> 52) & 0x7FF) - 1023;
    if (e >= 0 || e < -52) return -1;
    const uint64_t m = (b & ((1ULL << 52) - 1)) | (1ULL << 52);
    if (m & ((1ULL << -e) - 1)) return -1;
    return (int64_t)(m >> -e);
}
/* fill the y/z splits a zero input coordinate uses (the reference computes the same values per sample);
 * H is MgLattice or any header with the same field names; dbl: a double-branch world's lattice (the
 * fixed-point smoothsteps), else the float branch's */
template <typename H>
__device__ __forceinline__ void lattice_header(H &L, bool dbl) {
    L.iy = ifloor(L.oy);
    L.iz = ifloor(L.oz);
    L.fyd = L.oy - (double)L.iy;
    L.fzd = L.oz - (double)L.iz;
    L.uyd = fade_h<double>(L.fyd);
    L.uzd = fade_h<double>(L.fzd);
    L.Fy = fixed52(L.fyd);
    L.Fz = fixed52(L.fzd);
    if (dbl) {
        L.z0.q.uy = L.Fy < 0 ? 0 : fadeq(L.Fy << (MG_Q - 52));
        L.z0.q.uz = L.Fz < 0 ? 0 : fadeq(L.Fz << (MG_Q - 52));
    } else {
        L.z0.f.fy = (float)L.fyd;
        L.z0.f.fz = (float)L.fzd;
        L.z0.f.uy = fade_h<float>(L.z0.f.fy);
        L.z0.f.uz = fade_h<float>(L.z0.f.fz);
    }
}
/* the header's 16-byte words (the permutation follows them) */
#define MG_LAT_HDR_WORDS ((int)(offsetof(MgLattice, p) / 16))

/* ------------------------------------------------------------------ Perlin octave (shared lattice math) */
/* gradient dot with SimplexNoise.GRADIENT[h & 15]: every vector has two +-1 components, so the dot is a
 * signed sum of two coordinates.  (It can differ from g.x*x + g.y*y + g.z*z only in the sign of an
 * exactly-zero result, which no later step of the path can observe: the layer sum starts at +0.) */
template <typename T>
__device__ __forceinline__ T gdot(int h, T x, T y, T z) {
    h &= 15;
    T u = h < 8 ? x : y;
    T v = h < 4 ? y : ((h == 12 || h == 14) ? x : z);
    return ((h & 1) ? -u : u) + ((h & 2) ? -v : v);
}
/* The float branch (bound by the integer ALU pipe) takes the vector from a 256-byte table through L1 and
 * forms the dot on the FMA pipe: gy*y is exact, fma(gx, x, .) and fma(gz, z, .) each round at most once
 * and, with exactly two non-zero components, exactly one of them rounds -- the reference's one rounded
 * sum of two exact products (up to the sign of an exactly-zero result, as above). */
__device__ const float4 kGradF[16] = {{1, 1, 0, 0},  {-1, 1, 0, 0}, {1, -1, 0, 0}, {-1, -1, 0, 0}, {1, 0, 1, 0},  {-1, 0, 1, 0},
                                      {1, 0, -1, 0}, {-1, 0, -1, 0}, {0, 1, 1, 0},  {0, -1, 1, 0},  {0, 1, -1, 0}, {0, -1, -1, 0},
                                      {1, 1, 0, 0},  {0, -1, 1, 0},  {-1, 1, 0, 0}, {0, -1, -1, 0}};
template <>
__device__ __forceinline__ float gdot<float>(int h, float x, float y, float z) {
    const float4 g = __ldg(&kGradF[h & 15]);
    return __fmaf_rn(g.z, z, __fmaf_rn(g.x, x, g.y * y));
}
template <typename T>
__device__ __forceinline__ T fade(T t) {
    return t * t * t * (t * (t * (T)6 - (T)15) + (T)10);
}
template <typename T>
__device__ __forceinline__ T lerp(T t, T a, T b) { return a + t * (b - a); }

/* Permutation access: a plain 256-byte table, or a thread's own table in the interleaved shared layout
 * (byte i of thread t in byte i & 3 of word [i >> 2][t]; every access of a thread hits bank t % 32). */
struct PlainPerm {
    const uint8_t *p;
    __device__ __forceinline__ int operator()(int i) const { return p[i & 255]; }
};
template <int NT>
struct IlvPerm {
    const uint8_t *base; /* start of the [64][NT] word array */
    int t;
    __device__ __forceinline__ int operator()(int i) const {
        i &= 255;
        return base[((((i >> 2) * NT) + t) << 2) | (i & 3)];
    }
};

/* ImprovedNoise.sampleAndLerp with split coordinates (engine/mc_noise.h:54-75 / 90-110); g* = f* - 1 and
 * u, v, w = fade(fx), fade(fy), fade(fz) are passed in so that a coordinate split once per lattice (the
 * zero input coordinate) is not recomputed per sample. */
template <typename T, typename P>
__device__ __forceinline__ T octave_q(const P &p, int ix, T fx, int iy, T fy, T gy, T v, int iz, T fz, T gz, T w) {
    int a = p(ix), b = p(ix + 1);
    int aa = p(a + iy), ab = p(a + iy + 1);
    int ba = p(b + iy), bb = p(b + iy + 1);
    T gx = fx - (T)1;
    T c000 = gdot<T>(p(aa + iz), fx, fy, fz);
    T c100 = gdot<T>(p(ba + iz), gx, fy, fz);
    T c010 = gdot<T>(p(ab + iz), fx, gy, fz);
    T c110 = gdot<T>(p(bb + iz), gx, gy, fz);
    T c001 = gdot<T>(p(aa + iz + 1), fx, fy, gz);
    T c101 = gdot<T>(p(ba + iz + 1), gx, fy, gz);
    T c011 = gdot<T>(p(ab + iz + 1), fx, gy, gz);
    T c111 = gdot<T>(p(bb + iz + 1), gx, gy, gz);
    T u = fade<T>(fx);
    return lerp<T>(w, lerp<T>(v, lerp<T>(u, c000, c100), lerp<T>(u, c010, c110)),
                   lerp<T>(v, lerp<T>(u, c001, c101), lerp<T>(u, c011, c111)));
}
template <typename T, typename P>
__device__ __forceinline__ T octave_p(const P &p, int ix, T fx, int iy, T fy, int iz, T fz) {
    return octave_q<T>(p, ix, fx, iy, fy, fy - (T)1, fade<T>(fy), iz, fz, fz - (T)1, fade<T>(fz));
}
/* input coordinate y (resp. z) zero: its split comes from the lattice header */
template <typename T> struct Hdr;
template <> struct Hdr<float> {
    template <typename H> __device__ static float fy(const H &h) { return h.z0.f.fy; }
    template <typename H> __device__ static float fz(const H &h) { return h.z0.f.fz; }
    template <typename H> __device__ static float gy(const H &h) { return h.z0.f.fy - 1.0f; }
    template <typename H> __device__ static float gz(const H &h) { return h.z0.f.fz - 1.0f; }
    template <typename H> __device__ static float uy(const H &h) { return h.z0.f.uy; }
    template <typename H> __device__ static float uz(const H &h) { return h.z0.f.uz; }
};
template <> struct Hdr<double> {
    template <typename H> __device__ static double fy(const H &h) { return h.fyd; }
    template <typename H> __device__ static double fz(const H &h) { return h.fzd; }
    template <typename H> __device__ static double gy(const H &h) { return h.fyd - 1.0; }
    template <typename H> __device__ static double gz(const H &h) { return h.fzd - 1.0; }
    template <typename H> __device__ static double uy(const H &h) { return h.uyd; }
    template <typename H> __device__ static double uz(const H &h) { return h.uzd; }
};
template <typename T, typename P, typename H>
__device__ __forceinline__ T octave_y0(const P &p, const H &h, int ix, T fx, int iz, T fz) {
    using Q = Hdr<T>;
    return octave_q<T>(p, ix, fx, h.iy, Q::fy(h), Q::gy(h), Q::uy(h), iz, fz, fz - (T)1, fade<T>(fz));
}
template <typename T, typename P, typename H>
__device__ __forceinline__ T octave_z0(const P &p, const H &h, int ix, T fx, int iy, T fy) {
    using Q = Hdr<T>;
    return octave_q<T>(p, ix, fx, iy, fy, fy - (T)1, fade<T>(fy), h.iz, Q::fz(h), Q::gz(h), Q::uz(h));
}
/* Double branch in 2^-52 fixed point.  When the three fractions are multiples of 2^-52 (always, once the
 * coordinate split is exact and the sum has magnitude >= 1), fx - 1 and the eight gradient sums are exact
 * in double, so they are formed as integers; the first lerp level's differences b - a are rounded to
 * double once, exactly as the reference's subtraction rounds them.  Only the smoothsteps and the rounded
 * lerp products and sums stay on the FP64 pipe (36 instead of 50 FP64 operations per octave sample).
 * Integer and FP64 results differ at most in the sign of an exactly-zero corner value, which no later
 * step observes (as for gdot). */
__device__ const int4 kGradI[16] = {{1, 1, 0, 0},  {-1, 1, 0, 0}, {1, -1, 0, 0}, {-1, -1, 0, 0}, {1, 0, 1, 0},  {-1, 0, 1, 0},
                                    {1, 0, -1, 0}, {-1, 0, -1, 0}, {0, 1, 1, 0},  {0, -1, 1, 0},  {0, 1, -1, 0}, {0, -1, -1, 0},
                                    {1, 1, 0, 0},  {0, -1, 1, 0},  {-1, 1, 0, 0}, {0, -1, -1, 0}};
/* the vector from the table, the dot as 64-bit products with the small components (the integer
 * multiply-add pipe) instead of 64-bit selects and negations on the ALU pipe; exact either way */
__device__ __forceinline__ int64_t gdot_i(int h, int64_t x, int64_t y, int64_t z) {
    const int4 g = __ldg(&kGradI[h & 15]);
    return x * (int64_t)g.x + y * (int64_t)g.y + z * (int64_t)g.z;
}
/* lerp(u, a, b) = a + u * (b - a) for a = A * 2^-52, b = B * 2^-52, scaled by 2^52: the hardware's
 * round-to-nearest-even conversions of A (|A| <= 2^53: exact) and of B - A (|B - A| < 2^55: rounded as the
 * reference's subtraction b - a rounds), then the product and the sum.  Scaling by a power of two commutes
 * with every rounding while the values stay normal (here they are integers or products of a smoothstep
 * above 2^-160 with them), so the scaled lerps give 2^52 times the reference's lerps exactly. */
__device__ __forceinline__ double fix_lerp52(double u, int64_t A, int64_t B) {
    return __ll2double_rn(A) + u * __ll2double_rn(B - A);
}
/* the same with the smoothstep u of the x fraction given (a precomputed split); the second and third lerp
 * levels run on the scaled values and one product by 2^-52 (exact) undoes the scale */
template <typename P>
__device__ __forceinline__ double octave_dfix_u(const P &p, int ix, int64_t FX, double u, int iy, int64_t FY, double v,
                                                int iz, int64_t FZ, double w) {
    const int64_t ONE = 1LL << 52;
    const int a = p(ix), b = p(ix + 1);
    const int aa = p(a + iy), ab = p(a + iy + 1);
    const int ba = p(b + iy), bb = p(b + iy + 1);
    const int64_t GX = FX - ONE, GY = FY - ONE, GZ = FZ - ONE;
    const double x00 = fix_lerp52(u, gdot_i(p(aa + iz), FX, FY, FZ), gdot_i(p(ba + iz), GX, FY, FZ));
    const double x10 = fix_lerp52(u, gdot_i(p(ab + iz), FX, GY, FZ), gdot_i(p(bb + iz), GX, GY, FZ));
    const double x01 = fix_lerp52(u, gdot_i(p(aa + iz + 1), FX, FY, GZ), gdot_i(p(ba + iz + 1), GX, FY, GZ));
    const double x11 = fix_lerp52(u, gdot_i(p(ab + iz + 1), FX, GY, GZ), gdot_i(p(bb + iz + 1), GX, GY, GZ));
    return lerp<double>(w, lerp<double>(v, x00, x10), lerp<double>(v, x01, x11)) * 0x1.0p-52;
}
template <typename P>
__device__ __forceinline__ double octave_dfix(const P &p, int ix, double fx, int64_t FX, int iy, int64_t FY, double v,
                                              int iz, int64_t FZ, double w) {
    return octave_dfix_u(p, ix, FX, fade<double>(fx), iy, FY, v, iz, FZ, w);
}
/* the plain double octave, for a fraction that is not a multiple of 2^-52 (rare): out of line for a plain
 * table, inline for the interleaved shared layout */
static __device__ __noinline__ double octave_d_plain(const uint8_t *p, int ix, double fx, int iy, double fy, double v,
                                                     int iz, double fz, double w) {
    return octave_q<double>(PlainPerm{p}, ix, fx, iy, fy, fy - 1.0, v, iz, fz, fz - 1.0, w);
}
template <typename P>
__device__ __forceinline__ double octave_d_rare(const P &p, int ix, double fx, int iy, double fy, double v, int iz,
                                                double fz, double w) {
    return octave_q<double>(p, ix, fx, iy, fy, fy - 1.0, v, iz, fz, fz - 1.0, w);
}
__device__ __forceinline__ double octave_d_rare(const PlainPerm &p, int ix, double fx, int iy, double fy, double v, int iz,
                                                double fz, double w) {
    return octave_d_plain(p.p, ix, fx, iy, fy, v, iz, fz, w);
}
/* double octave with input y (resp. z) zero: fixed point when every fraction allows it */
template <typename P, typename H>
__device__ __forceinline__ double octave_d_y0(const P &p, const H &h, int ix, double fx, int64_t FX, int iz, double fz,
                                              int64_t FZ) {
    const double w = fade<double>(fz);
    if ((FX | FZ | h.Fy) >= 0) return octave_dfix(p, ix, fx, FX, h.iy, h.Fy, h.uyd, iz, FZ, w);
    return octave_d_rare(p, ix, fx, h.iy, h.fyd, h.uyd, iz, fz, w);
}
template <typename P, typename H>
__device__ __forceinline__ double octave_d_z0(const P &p, const H &h, int ix, double fx, int64_t FX, int iy, double fy,
                                              int64_t FY) {
    const double v = fade<double>(fy);
    if ((FX | FY | h.Fz) >= 0) return octave_dfix(p, ix, fx, FX, iy, FY, v, h.iz, h.Fz, h.uzd);
    return octave_d_rare(p, ix, fx, iy, fy, v, h.iz, h.fzd, h.uzd);
}
template <typename T>
__device__ __forceinline__ T octave(const uint8_t *__restrict__ p, int ix, T fx, int iy, T fy, int iz, T fz) {
    return octave_p<T>(PlainPerm{p}, ix, fx, iy, fy, iz, fz);
}

/* mulq_u for a non-negative weight t and a signed value s: the unsigned high product of t and s's two's
 * complement bits is the signed one plus t when s < 0 (one correction instead of a signed product's two) */
__device__ __forceinline__ int64_t mulq_us(int64_t t, int64_t s) {
    const uint64_t hi = __umul64hi((uint64_t)t, (uint64_t)s) - (s < 0 ? (uint64_t)t : 0ULL);
    const uint64_t lo = (uint64_t)t * (uint64_t)s;
    return (int64_t)((hi << (64 - MG_Q)) | (lo >> MG_Q));
}
/* the octave in the 59-bit fixed point of mulq_u / fadeq (the weights t are smoothsteps in [0, 1]) */
__device__ __forceinline__ int64_t lerpq(int64_t t, int64_t a, int64_t b) { return a + mulq_us(t, b - a); }
/* fractions X, Y, Z and smoothsteps V, W (of Y, Z) in the fixed point */
template <typename P>
__device__ __forceinline__ int64_t octave_qfix(const P &p, int ix, int64_t X, int iy, int64_t Y, int64_t V, int iz,
                                               int64_t Z, int64_t W) {
    const int64_t ONE = 1LL << MG_Q;
    const int a = p(ix), b = p(ix + 1);
    const int aa = p(a + iy), ab = p(a + iy + 1);
    const int ba = p(b + iy), bb = p(b + iy + 1);
    const int64_t GX = X - ONE, GY = Y - ONE, GZ = Z - ONE;
    const int64_t U = fadeq(X);
    const int64_t x00 = lerpq(U, gdot_i(p(aa + iz), X, Y, Z), gdot_i(p(ba + iz), GX, Y, Z));
    const int64_t x10 = lerpq(U, gdot_i(p(ab + iz), X, GY, Z), gdot_i(p(bb + iz), GX, GY, Z));
    const int64_t x01 = lerpq(U, gdot_i(p(aa + iz + 1), X, Y, GZ), gdot_i(p(ba + iz + 1), GX, Y, GZ));
    const int64_t x11 = lerpq(U, gdot_i(p(ab + iz + 1), X, GY, GZ), gdot_i(p(bb + iz + 1), GX, GY, GZ));
    return lerpq(W, lerpq(V, x00, x10), lerpq(V, x01, x11));
}

/* 26.3 PerlinNoise.wrap: identity inside (-2^24, 2^24) (engine/mc_noise.h:86-89) */
__device__ __forceinline__ double wrap_new(double x) {
    const double lim = 16777215.999999998;
    if (x >= -lim && x < lim) return x;
    return x - (double)lfloor(x / 33554432.0 + 0.5) * 33554432.0;
}
/* 26.1/26.2 PerlinNoise.wrap (engine/mc_noise.h:76-77); exact identity for |x| < 2^23 */
__device__ __forceinline__ double wrap_old(double x) {
    if (fabs(x) < 8388608.0) return x;
    return x - (double)lfloor(x / 33554432.0 + 0.5) * 33554432.0;
}
/* One input coordinate -> lattice cell and fraction, as the reference computes it (all in double). */
__device__ __forceinline__ void split_f_plain(double v, double off, int &i, float &f) {
    double s = wrap_new(v) + off;
    i = ifloor(s);
    f = (float)(s - (double)i);
}
__device__ __forceinline__ void split_d_plain(double v, double off, int &i, double &f) {
    double s = wrap_old(v) + off;
    i = ifloor(s);
    f = s - (double)i;
}

/* fb * 2^-sh rounded to nearest-even float (fb < 2^53; the result exponent must be >= -126): the hardware
 * conversion of fb rounds to nearest-even, and the power-of-two scaling of a normal result is exact (an
 * exponent subtraction), so this is the rounded product.  One conversion on the XU pipe instead of about
 * fifteen integer operations of a rounding emulation on the ALU pipe, the float branch's busiest. */
__device__ __forceinline__ float scaled_to_f32(uint64_t fb, int sh) {
    if (fb == 0) return 0.0f;
    return __int_as_float(__float_as_int(__ull2float_rn(fb)) - (sh << 23));
}
/* fb * 2^-sh exactly as a double (fb < 2^53) */
__device__ __forceinline__ double scaled_to_f64(uint64_t fb, int sh) {
    if (fb == 0) return 0.0;
    const int L = 64 - __clzll((long long)fb);
    const uint64_t mant = fb << (53 - L);
    return __longlong_as_double((long long)(((uint64_t)(L - 1 - sh + 1023) << 52) | (mant & ((1ULL << 52) - 1))));
}

/* The same split for v = x * 2^k, exactly equal to split_*_plain(x * f, off) with f = 2^k, but with one
 * FP64-pipe operation (the rounded add s = v + off) instead of eight: GB300 runs FP64 at about 1/70 of the
 * FP32 rate.  x * 2^k is an exponent add; the wrap is the identity for |v| < 2^23; floor(s) and the exact
 * fraction s - floor(s) come from the bits of s, and the float fraction is rounded to nearest-even in
 * integer arithmetic.  Cases outside those bounds (|v| >= 2^23, s in (-1, 0), tiny s) take the plain path. */
template <bool F32>
__device__ __forceinline__ bool split_bits(double s, int &i, float &ff, double &fd) {
    const uint64_t b = (uint64_t)__double_as_longlong(s);
    const int ebits = (int)((b >> 52) & 0x7FF);
    const bool neg = (b >> 63) != 0;
    if (ebits == 0) {
        if ((b << 1) != 0) return false; /* subnormal */
        i = 0;                            /* +-0: floor 0, fraction s - 0 = s */
        ff = neg ? -0.0f : 0.0f;
        fd = s;
        return true;
    }
    const int e = ebits - 1023;
    if (e > 30) return false;
    const uint64_t m = (b & ((1ULL << 52) - 1)) | (1ULL << 52);
    if (!neg) {
        if (e >= 0) {
            const int sh = 52 - e;
            i = (int)(m >> sh);
            const uint64_t fb = m & ((1ULL << sh) - 1);
            if (F32) ff = scaled_to_f32(fb, sh);
            else fd = scaled_to_f64(fb, sh);
        } else {
            if (F32 && e < -126) return false;
            i = 0;
            if (F32) ff = scaled_to_f32(m, 52 - e);
            else fd = s;
        }
        return true;
    }
    if (e < 0) return false; /* s in (-1, 0): the reference's s - floor(s) rounds */
    const int sh = 52 - e;
    const uint64_t ip = m >> sh, fb = m & ((1ULL << sh) - 1);
    if (fb == 0) {
        i = -(int)ip;
        ff = 0.0f;
        fd = 0.0;
    } else {
        i = -(int)ip - 1;
        if (F32) ff = scaled_to_f32((1ULL << sh) - fb, sh);
        else fd = scaled_to_f64((1ULL << sh) - fb, sh);
    }
    return true;
}
/* x * 2^k by an exponent add when x is a normal double and the product stays below 2^23 in magnitude */
__device__ __forceinline__ bool scale_small(double x, int k, double &v) {
    const uint64_t b = (uint64_t)__double_as_longlong(x);
    const int ebits = (int)((b >> 52) & 0x7FF);
    if (ebits == 0) {
        if ((b << 1) != 0) return false;
        v = x; /* +-0 */
        return true;
    }
    const int ne = ebits + k;
    if (ne <= 0 || ne >= 1023 + 23) return false;
    v = __longlong_as_double((long long)(b + ((uint64_t)(int64_t)k << 52)));
    return true;
}
/* The plain splits (|v| >= 2^23, s in (-1, 0), tiny s: rare) carry the wrap's double division; one
 * out-of-line copy keeps them out of the octave loops' hot code. */
struct SplitF {
    int i;
    float f;
};
struct SplitD {
    int i;
    double f;
    int64_t F;
};
static __device__ __noinline__ SplitF split_f_slow(double v, double off) {
    SplitF r;
    split_f_plain(v, off, r.i, r.f);
    return r;
}
static __device__ __noinline__ SplitD split_d_slow(double v, double off) {
    SplitD r;
    split_d_plain(v, off, r.i, r.f);
    r.F = fixed52(r.f);
    return r;
}
__device__ __forceinline__ void split_fk(double x, double f, int k, double off, int &i, float &fr) {
    double v, fd;
    if (scale_small(x, k, v) && split_bits<true>(v + off, i, fr, fd)) return;
    const SplitF r = split_f_slow(x * f, off);
    i = r.i;
    fr = r.f;
}
/* Double-branch split of s = v + off that also gives the fraction in units of 2^-52 (F, or -1 when the
 * fraction is not a multiple of 2^-52); false where the plain arithmetic must be used. */
__device__ __forceinline__ bool split_bits_d(double s, int &i, double &fd, int64_t &F) {
    const uint64_t b = (uint64_t)__double_as_longlong(s);
    const int ebits = (int)((b >> 52) & 0x7FF);
    const bool neg = (b >> 63) != 0;
    if (ebits == 0) {
        if ((b << 1) != 0) return false; /* subnormal */
        i = 0;                            /* +-0: floor 0, fraction s - 0 = s */
        fd = s;
        F = 0;
        return true;
    }
    const int e = ebits - 1023;
    if (e > 30) return false;
    const uint64_t m = (b & ((1ULL << 52) - 1)) | (1ULL << 52);
    if (!neg) {
        if (e >= 0) {
            const int sh = 52 - e;
            const uint64_t fb = m & ((1ULL << sh) - 1);
            i = (int)(m >> sh);
            fd = scaled_to_f64(fb, sh);
            F = (int64_t)(fb << e);
        } else {
            i = 0;
            fd = s;
            F = fixed52(s);
        }
        return true;
    }
    if (e < 0) return false; /* s in (-1, 0): the reference's s - floor(s) rounds */
    const int sh = 52 - e;
    const uint64_t ip = m >> sh, fb = m & ((1ULL << sh) - 1);
    if (fb == 0) {
        i = -(int)ip;
        fd = 0.0;
        F = 0;
    } else {
        const uint64_t r = (1ULL << sh) - fb;
        i = -(int)ip - 1;
        fd = scaled_to_f64(r, sh);
        F = (int64_t)(r << e);
    }
    return true;
}
__device__ __forceinline__ void split_dk(double x, double f, int k, double off, int &i, double &fr, int64_t &F) {
    double v;
    if (scale_small(x, k, v) && split_bits_d(v + off, i, fr, F)) return;
    const SplitD r = split_d_slow(x * f, off);
    i = r.i;
    fr = r.f;
    F = r.F;
}

/* Octave of lattice L with input (a*f, 0, b*f) (z0 false) or (a*f, b*f, 0) (z0 true); the zero coordinate
 * uses the table's split.  One copy serves both forms (the zero coordinate's values are selected), which
 * keeps the noise loops' code small. */
__device__ __forceinline__ float oct_f(const MgLattice *__restrict__ L, double a, double b, double f, int k, bool z0) {
    int ia, ib;
    float fa, fb;
    split_fk(a, f, k, L->ox, ia, fa);
    split_fk(b, f, k, z0 ? L->oy : L->oz, ib, fb);
    const int i0 = z0 ? L->iz : L->iy;
    const float f0 = z0 ? L->z0.f.fz : L->z0.f.fy, u0 = z0 ? L->z0.f.uz : L->z0.f.uy, ub = fade<float>(fb);
    const int iy = z0 ? ib : i0, iz = z0 ? i0 : ib;
    const float fy = z0 ? fb : f0, fz = z0 ? f0 : fb, v = z0 ? ub : u0, w = z0 ? u0 : ub;
    return octave_q<float>(PlainPerm{L->p}, ia, fa, iy, fy, fy - 1.0f, v, iz, fz, fz - 1.0f, w);
}
__device__ __forceinline__ double oct_d(const MgLattice *__restrict__ L, double a, double b, double f, int k, bool z0) {
    int ia, ib;
    double fa, fb;
    int64_t FA, FB;
    split_dk(a, f, k, L->ox, ia, fa, FA);
    split_dk(b, f, k, z0 ? L->oy : L->oz, ib, fb, FB);
    const int i0 = z0 ? L->iz : L->iy;
    const int64_t F0 = z0 ? L->Fz : L->Fy;
    const double f0 = z0 ? L->fzd : L->fyd, u0 = z0 ? L->uzd : L->uyd, ub = fade<double>(fb);
    const int iy = z0 ? ib : i0, iz = z0 ? i0 : ib;
    const double v = z0 ? ub : u0, w = z0 ? u0 : ub;
    if ((FA | FB | F0) >= 0) return octave_dfix(PlainPerm{L->p}, ia, fa, FA, iy, z0 ? FB : F0, v, iz, z0 ? F0 : FB, w);
    return octave_d_plain(L->p, ia, fa, iy, z0 ? fb : f0, v, iz, z0 ? f0 : fb, w);
}

/* ------------------------------------------------------------------ NormalNoise (engine/mc_noise.h:285-324)
 * Not inlined: a climate evaluation calls them six times per branch, and the grid kernels evaluate the
 * climate at several sites (direct and along a tie chain); one out-of-line copy each keeps the kernels'
 * hot code within the instruction cache, at the cost of a call per noise (2 x 2..9 octaves).
 * Every NormalNoise on the biome path has one input coordinate equal to zero: the five climate noises
 * and the Nether noises take (x, 0, z), ShiftA (x, 0, z), ShiftB (z, x, 0).  The second stack's input
 * x*(f*c) equals (x*c)*f exactly (f = 2^k), so xc = x*c is formed once per point. */
/* float branch, non-legacy (interleaved first_k, second_k); input (a, 0, b), or (a, b, 0) when z0 */
static __device__ __noinline__ float nn_f(const MgNoise &N, const MgLattice *__restrict__ T, double a, double b,
                                          double ac, double bc, bool z0) {
    float acc = 0.0f;
    const MgLattice *A = T + N.base, *B = A + N.nlev;
    /* one octave per step, first and second stack of each level in turn (the reference's order): one copy of
     * the octave code (the batch kernel runs every code path's tiles side by side, so all of their hot code
     * shares the instruction cache) */
#pragma unroll 1
    for (int j = 0; j < 2 * N.nlev; j++) {
        const int k = j >> 1, st = j & 1;
        acc += N.amp_f[k] * oct_f((st ? B : A) + k, st ? ac : a, st ? bc : b, N.freq[k], N.fexp[k], z0);
    }
    return acc;
}
__device__ __forceinline__ float nn_f_y0(const MgNoise &N, const MgLattice *__restrict__ T, double x, double z,
                                         double xc, double zc) {
    return nn_f(N, T, x, z, xc, zc, false);
}
__device__ __forceinline__ float nn_f_z0(const MgNoise &N, const MgLattice *__restrict__ T, double x, double y,
                                         double xc, double yc) {
    return nn_f(N, T, x, y, xc, yc, true);
}
/* float branch, legacy Nether form (whole first stack, then whole second stack) */
static __device__ __noinline__ float nn_f_legacy_y0(const MgNoise &N, const MgLattice *__restrict__ T, double x, double z,
                                                double xc, double zc) {
    float acc = 0.0f;
    const MgLattice *A = T + N.base, *B = A + N.nlev;
    for (int k = 0; k < N.nlev; k++) acc += N.amp_f[k] * oct_f(A + k, x, z, N.freq[k], N.fexp[k], false);
    for (int k = 0; k < N.nlev; k++) acc += N.amp_f[k] * oct_f(B + k, xc, zc, N.freq[k], N.fexp[k], false);
    return acc;
}
/* double branch: (first + second) * valueFactor; input (a, 0, b), or (a, b, 0) when z0 */
static __device__ __noinline__ double nn_d(const MgNoise &N, const MgLattice *__restrict__ T, double a, double b,
                                           double ac, double bc, bool z0) {
    double s[2] = {0.0, 0.0};
    const MgLattice *A = T + N.base;
    /* the two stacks' sums advance together in one loop (one copy of the octave code); each keeps its order */
    for (int j = 0; j < 2 * N.nlev; j++) {
        const int k = j >> 1, st = j & 1;
        const double o = oct_d(A + st * N.nlev + k, st ? ac : a, st ? bc : b, N.freq[k], N.fexp[k], z0);
        const double t = N.amp_d[k] * o * N.vf_d[k];
        if (st) s[1] += t;
        else s[0] += t;
    }
    return (s[0] + s[1]) * N.vfac;
}
__device__ __forceinline__ double nn_d_y0(const MgNoise &N, const MgLattice *__restrict__ T, double x, double z,
                                          double xc, double zc) {
    return nn_d(N, T, x, z, xc, zc, false);
}
__device__ __forceinline__ double nn_d_z0(const MgNoise &N, const MgLattice *__restrict__ T, double x, double y,
                                          double xc, double yc) {
    return nn_d(N, T, x, y, xc, yc, true);
}

/* double branch, screened: the NormalNoise value in fixed point (every level's amplitude, level value
 * factor and the noise's value factor folded into N.cq), in units of 2^-59; input (a, 0, b) (Z0 false:
 * the climate noises and ShiftA) or (a, b, 0) (Z0 true: ShiftB), with ac, bc the second stack's inputs.
 * The zero coordinate's split and smoothstep come from the lattice header.  MG_QFAIL when a fraction of the
 * input split is not a multiple of 2^-52 (the exact path handles those); |value| < 15 * 2^59 otherwise. */
#define MG_QFAIL INT64_MIN
template <bool Z0>
static __device__ __noinline__ int64_t nn_q(const MgNoise &N, const MgLattice *__restrict__ T, double a, double b,
                                            double ac, double bc) {
    int64_t acc = 0, lev = 0;
    const MgLattice *A = T + N.base;
    /* one loop over both stacks' levels, one copy of the octave code (the kernels' hot code stays small);
     * a level's two octaves are summed before the product with the level's constant (the sum is exact, so
     * its order is free) */
    for (int j = 0; j < 2 * N.nlev; j++) {
        const int k = j >> 1, st = j & 1;
        const MgLattice *L = A + st * N.nlev + k;
        const double f = N.freq[k];
        int ia, ib;
        double fa, fb;
        int64_t FA, FB;
        split_dk(st ? ac : a, f, N.fexp[k], L->ox, ia, fa, FA);
        split_dk(st ? bc : b, f, N.fexp[k], Z0 ? L->oy : L->oz, ib, fb, FB);
        const int64_t F0 = Z0 ? L->Fz : L->Fy;
        if ((FA | FB | F0) < 0) return MG_QFAIL;
        const int64_t XA = FA << (MG_Q - 52), XB = FB << (MG_Q - 52), X0 = F0 << (MG_Q - 52);
        lev += Z0 ? octave_qfix(PlainPerm{L->p}, ia, XA, ib, XB, fadeq(XB), L->iz, X0, L->z0.q.uz)
                  : octave_qfix(PlainPerm{L->p}, ia, XA, L->iy, X0, L->z0.q.uy, ib, XB, fadeq(XB));
        if (st) {
            const int64_t c = N.cq[k], m = mulq_us(c < 0 ? -c : c, lev);
            acc += c < 0 ? -m : m;
            lev = 0;
        }
    }
    return acc;
}
/* The 32-bit screened form of nn_q (input (a, 0, b)), for a noise whose value is only quantised (the double
 * branch's Nether noises: their floats feed nothing but quantize, whose steps of 1e-4 need far less precision
 * than a float's rounding): the octaves in 28-bit fixed point (values in units of 2^-28 in
 * int32, below 8 in magnitude), the smoothstep weights in units of 2^-31, every lerp one 32 x 32-bit product
 * where nn_q's 59-bit form takes a 64 x 64-bit one, and the levels' constants N.c31 (units of 2^-31) bring
 * the sum to nn_q's units of 2^-59.  Within N.fix_eq32 units of the reference's double value (the host's
 * bound); MG_QFAIL as nn_q. */
/* smoothstep of a fraction t (units of 2^-32), in units of 2^-31: t^3 (6t^2 - 15t + 10) with t^3 truncated
 * once from the exact t^2, the factor (in [1, 10]) from t^2 truncated, and their product truncated */
__device__ __forceinline__ int32_t fade31(uint32_t t) {
    const uint64_t t2w = (uint64_t)t * t;
    const uint32_t t2 = (uint32_t)(t2w >> 32);
    const uint32_t t3 = (uint32_t)(((uint64_t)t2 * t + (((uint64_t)(uint32_t)t2w * t) >> 32)) >> 32);
    const int64_t p = (10LL << 32) + 6 * (int64_t)t2 - 15 * (int64_t)t; /* > 2^32 - 7: positive */
    const uint32_t f = (uint32_t)(((uint64_t)t3 * (uint32_t)p) >> 32) + t3 * (uint32_t)(p >> 32);
    return (int32_t)(f >> 1);
}
/* a + w (b - a) for a weight w in [0, 1) (units of 2^-31), floored */
__device__ __forceinline__ int32_t lerp28(int32_t w, int32_t a, int32_t b) {
    return a + (int32_t)(((int64_t)w * (int64_t)(b - a)) >> 31);
}
__device__ __forceinline__ int32_t gdot28(int h, int32_t x, int32_t y, int32_t z) {
    const int4 g = __ldg(&kGradI[h & 15]);
    return x * g.x + y * g.y + z * g.z;
}
/* fractions X, Y, Z (units of 2^-28) and weights U, V, W (of X, Y, Z; units of 2^-31) */
template <typename P>
__device__ __forceinline__ int32_t octave_q28(const P &p, int ix, int32_t X, int32_t U, int iy, int32_t Y, int32_t V,
                                              int iz, int32_t Z, int32_t W) {
    const int32_t ONE = 1 << 28;
    const int a = p(ix), b = p(ix + 1);
    const int aa = p(a + iy), ab = p(a + iy + 1);
    const int ba = p(b + iy), bb = p(b + iy + 1);
    const int32_t GX = X - ONE, GY = Y - ONE, GZ = Z - ONE;
    const int32_t x00 = lerp28(U, gdot28(p(aa + iz), X, Y, Z), gdot28(p(ba + iz), GX, Y, Z));
    const int32_t x10 = lerp28(U, gdot28(p(ab + iz), X, GY, Z), gdot28(p(bb + iz), GX, GY, Z));
    const int32_t x01 = lerp28(U, gdot28(p(aa + iz + 1), X, Y, GZ), gdot28(p(ba + iz + 1), GX, Y, GZ));
    const int32_t x11 = lerp28(U, gdot28(p(ab + iz + 1), X, GY, GZ), gdot28(p(bb + iz + 1), GX, GY, GZ));
    return lerp28(W, lerp28(V, x00, x10), lerp28(V, x01, x11));
}
static __device__ __noinline__ int64_t nn_q32(const MgNoise &N, const MgLattice *__restrict__ T, double a, double b,
                                              double ac, double bc) {
    int64_t acc = 0;
    int32_t lev = 0;
    const MgLattice *A = T + N.base;
    for (int j = 0; j < 2 * N.nlev; j++) {
        const int k = j >> 1, st = j & 1;
        const MgLattice *L = A + st * N.nlev + k;
        const double f = N.freq[k];
        int ia, ib;
        double fa, fb;
        int64_t FA, FB;
        split_dk(st ? ac : a, f, N.fexp[k], L->ox, ia, fa, FA);
        split_dk(st ? bc : b, f, N.fexp[k], L->oz, ib, fb, FB);
        if ((FA | FB | L->Fy) < 0) return MG_QFAIL;
        lev += octave_q28(PlainPerm{L->p}, ia, (int32_t)(FA >> 24), fade31((uint32_t)(FA >> 20)), L->iy,
                          (int32_t)(L->Fy >> 24), (int32_t)(L->z0.q.uy >> 28), ib, (int32_t)(FB >> 24),
                          fade31((uint32_t)(FB >> 20)));
        if (st) {
            acc += (int64_t)lev * N.c31[k];
            lev = 0;
        }
    }
    return acc;
}
/* the float the reference's double value rounds to, from a fixed-point approximation q (units of 2^-59)
 * within eq units of that value: true when every real in [q - eq, q + eq] 2^-59 rounds to the same float.
 * No FP64 pipe: the hardware's s64 -> f32 conversion rounds the integers q - eq and q + eq to
 * nearest (the scale 2^-59 is exact and keeps the order, so equal roundings of the two ends settle the
 * rounding of every value between them); the float is the rounded end times 2^-59 (normal: |q - eq| >= 1
 * when the ends agree, since eq > 0) */
__device__ __forceinline__ bool cast_settled_q(int64_t q, int64_t eq, float &f) {
    const float lo = __ll2float_rn(q - eq), hi = __ll2float_rn(q + eq);
    f = lo * 0x1.0p-59f;
    return lo == hi;
}

/* ------------------------------------------------------------------ offset spline (engine/mc_climate.h:38-66)
 * CubicSpline.Multipoint.apply, evaluated with an explicit stack instead of recursion. */
__device__ __forceinline__ float spline_eval(const MgSpline &S, const float co[4]) {
    if (S.root < 0) return S.cval[~S.root];
    struct Frame { int node, i; float in, y1; int state; };
    Frame st[MG_SPL_DEPTH];
    int sp = 0;
    float ret = 0.0f;
    st[0].node = S.root;
    st[0].state = 0;
    sp = 1;
    while (sp > 0) {
        Frame &f = st[sp - 1];
        int o = S.first[f.node], n = S.npts[f.node];
        if (f.state == 0) {
            float in = co[S.coord[f.node]];
            int lo = 0, len = n; /* Mth.binarySearch(0, n, i -> in < loc[i]) */
            while (len > 0) {
                int half = len >> 1, mid = lo + half;
                if (in < S.loc[o + mid]) len = half;
                else { lo = mid + 1; len -= half + 1; }
            }
            f.in = in;
            f.i = lo - 1;
            int c;
            if (f.i < 0 || f.i == n - 1) { f.state = 1; c = S.child[o + (f.i < 0 ? 0 : n - 1)]; }
            else { f.state = 2; c = S.child[o + f.i]; }
            if (c < 0) { ret = S.cval[~c]; continue; } /* constant child: deliver at once */
            st[sp].node = c;
            st[sp].state = 0;
            sp++;
            continue;
        }
        if (f.state == 1) { /* linear extension at the first or last point */
            int e = f.i < 0 ? 0 : n - 1;
            float d = S.der[o + e];
            ret = d == 0.0f ? ret : ret + d * (f.in - S.loc[o + e]);
            sp--;
            continue;
        }
        if (f.state == 2) { /* have y1, fetch y2 */
            f.y1 = ret;
            f.state = 3;
            int c = S.child[o + f.i + 1];
            if (c < 0) { ret = S.cval[~c]; continue; }
            st[sp].node = c;
            st[sp].state = 0;
            sp++;
            continue;
        }
        /* state 3: cubic Hermite interpolation */
        float x1 = S.loc[o + f.i], x2 = S.loc[o + f.i + 1];
        float t = (f.in - x1) / (x2 - x1);
        float d1 = S.der[o + f.i], d2 = S.der[o + f.i + 1];
        float y1 = f.y1, y2 = ret;
        float a = d1 * (x2 - x1) - (y2 - y1);
        float b = -d2 * (x2 - x1) + (y2 - y1);
        ret = lerp<float>(t, y1, y2) + t * (1.0f - t) * lerp<float>(t, a, b);
        sp--;
    }
    return ret;
}

/* ------------------------------------------------------------------ biome R-tree (engine/mc_biomes.h:31-62) */
__device__ __forceinline__ int32_t lo16(uint32_t w) { return (int32_t)(int16_t)(w & 0xFFFFu); }
__device__ __forceinline__ int32_t hi16(uint32_t w) { return (int32_t)w >> 16; }
__device__ __forceinline__ uint64_t dim_sq(int32_t t, int32_t lo, int32_t hi) {
    const int32_t x = max(max(t - hi, lo - t), 0);
    return (uint64_t)(uint32_t)x * (uint32_t)x;
}
/* squared distance of target t (6 quantised values; the offset coordinate is 0) to a node's box */
__device__ __forceinline__ uint64_t node_dist(const MgTreeNode &n, const int32_t *t) {
    const uint4 a = *reinterpret_cast<const uint4 *>(&n);                              /* lo[0..5], hi[0..1] */
    const uint4 b = *(reinterpret_cast<const uint4 *>(&n) + 1);                        /* hi[2..5], d7, links */
    uint64_t s = b.z; /* upper bounds are stored negated */
    s += dim_sq(t[0], lo16(a.x), -lo16(a.w));
    s += dim_sq(t[1], hi16(a.x), -hi16(a.w));
    s += dim_sq(t[2], lo16(a.y), -lo16(b.x));
    s += dim_sq(t[3], hi16(a.y), -hi16(b.x));
    s += dim_sq(t[4], lo16(a.z), -lo16(b.y));
    s += dim_sq(t[5], hi16(a.z), -hi16(b.y));
    return s;
}
/* Climate.RTree.SubTree.search, iterative: descend into a child iff its box distance is below the best
 * leaf distance so far; a leaf replaces the best iff strictly closer.  cand < 0: no candidate.  The
 * general form (explicit stack, 64-bit distances); tree_search below is the fast one. */
__device__ __forceinline__ int tree_search_stack(const MgTreeNode *__restrict__ T, const int32_t *t, int cand,
                                                 uint64_t &best) {
    int res = cand;
    best = cand < 0 ? ~0ULL : node_dist(T[cand], t);
    int stk_node[10];
    int stk_next[10];
    int sp = 0;
    stk_node[0] = 0;
    stk_next[0] = 0;
    sp = 1;
    while (sp > 0) {
        int nd = stk_node[sp - 1];
        int c = stk_next[sp - 1];
        int cnt = T[nd].count;
        if (c >= cnt) { sp--; continue; }
        stk_next[sp - 1] = c + 1;
        int ci = T[nd].first + c;
        uint64_t cd = node_dist(T[ci], t);
        if (cd < best) {
            if (T[ci].count == 0) { best = cd; res = ci; }
            else if (sp < 10) { stk_node[sp] = ci; stk_next[sp] = 0; sp++; }
        }
    }
    return res;
}
/* tree_search (no candidate) and whether a second leaf has the same fitness, in one traversal: children
 * are visited iff their box distance is <= the best so far, so every leaf at the final minimum is seen; the
 * first leaf to reach the minimum in tree order is kept -- the leaf tree_search returns, since no leaf
 * before it in tree order is as close -- and the leaves at the minimum are counted (capped at 2; the
 * tie test of libmcgen/src/biome.c:76-85). */
__device__ __forceinline__ int tree_search_tie_stack(const MgTreeNode *__restrict__ T, const int32_t *t, uint64_t &best,
                                                     bool &tied) {
    int stk_node[10], stk_next[10], sp = 1, res = -1, cnt = 0;
    best = ~0ULL;
    stk_node[0] = 0;
    stk_next[0] = 0;
    while (sp > 0) {
        const int nd = stk_node[sp - 1], c = stk_next[sp - 1];
        if (c >= T[nd].count) { sp--; continue; }
        stk_next[sp - 1] = c + 1;
        const int ci = T[nd].first + c;
        const uint64_t cd = node_dist(T[ci], t);
        if (cd > best) continue;
        if (T[ci].count == 0) {
            if (cd < best) { best = cd; res = ci; cnt = 1; }
            else if (cnt < 2) cnt++;
        } else if (sp < 10) {
            stk_node[sp] = ci; stk_next[sp] = 0; sp++;
        }
    }
    tied = cnt >= 2;
    return res;
}
/* The same searches with the traversal unrolled over the tree's levels (no stack in local memory: every
 * level's loop state stays in registers; leaves lie 3 to 5 levels below the root in every table, and
 * MG_RT_LEVELS + 1 levels below the root are unrolled) and 32-bit box distances from packed 16-bit pairs:
 * each dimension's distance is clamped at MG_RT_CLAMP, so six squares still fit in 32 bits, and the offset
 * term saturates below the initial bound.  A distance below MG_RT_CLAMP^2 is exact, and a node whose
 * distance was clamped or saturated is at least MG_RT_CLAMP^2 away, so whenever the final best distance is
 * below MG_RT_CLAMP^2 every comparison that decided the result was exact and the result is the 64-bit
 * search's; otherwise (or for a tree deeper than the unrolled levels, a tree whose bounds exceed the packed
 * range, or a target outside it) the stack form runs. */
#define MG_RT_CLAMP 26754
#define MG_RT_LEVELS 4
/* A target's coordinates as packed 16-bit pairs (t and -t): with every bound within +-12767 (the tree's
 * MG_TREE_PACKED flag) and |t| <= 20000, t - hi and lo - t fit 16 bits, and per pair of dimensions two
 * add-max instructions give max(lo - t, t - hi, 0) and one min the clamp. */
struct RtTarget {
    uint32_t p[3], n[3];
};
__device__ __forceinline__ uint32_t pack16(int32_t lo, int32_t hi) { return (uint32_t)(lo & 0xFFFF) | ((uint32_t)hi << 16); }
/* false when a coordinate is outside +-(32767 - MG_TREE_PACKED_BOUND) */
__device__ __forceinline__ bool rt_target(const int32_t *t, RtTarget &q) {
    const int32_t lim = 32767 - MG_TREE_PACKED_BOUND;
    bool ok = true;
    for (int k = 0; k < 6; k++) ok &= t[k] >= -lim && t[k] <= lim;
    for (int k = 0; k < 3; k++) {
        q.p[k] = pack16(t[2 * k], t[2 * k + 1]);
        q.n[k] = pack16(-t[2 * k], -t[2 * k + 1]);
    }
    return ok;
}
/* clamped squared distances of one pair of dimensions: lo = (lo_a, lo_b), nhi = (-hi_a, -hi_b) */
__device__ __forceinline__ uint32_t pair_sq(uint32_t lo, uint32_t nhi, uint32_t tp, uint32_t tn) {
    const uint32_t th = __viaddmax_s16x2(tp, nhi, 0x80008000u);   /* t - hi */
    uint32_t d = __viaddmax_s16x2_relu(lo, tn, th);                /* max(lo - t, t - hi, 0) */
    d = __vimin_s16x2_relu(d, (uint32_t)MG_RT_CLAMP * 0x10001u);   /* min(., clamp) */
    const uint32_t d0 = d & 0xFFFFu, d1 = d >> 16;
    return d0 * d0 + d1 * d1;
}
/* the node's clamped squared distance, the offset term saturating below the initial bound */
__device__ __forceinline__ uint32_t rt_dist(const uint4 &a, const uint4 &b, const RtTarget &q) {
    const uint32_t d = pair_sq(a.x, a.w, q.p[0], q.n[0]) + pair_sq(a.y, b.x, q.p[1], q.n[1]) +
                       pair_sq(a.z, b.y, q.p[2], q.n[2]);
    return d > 0xFFFFFFFEu - b.z ? 0xFFFFFFFEu : d + b.z;
}
struct RtState {
    uint32_t best;
    int res, cnt;
};
template <int D, bool TIE>
__device__ __forceinline__ bool rt_walk(const MgTreeNode *__restrict__ T, int first, int count, const RtTarget &q,
                                        RtState &s) {
    for (int ci = first; ci < first + count; ci++) {
        const uint4 a = *reinterpret_cast<const uint4 *>(T + ci);      /* lo[0..5], hi[0..1] */
        const uint4 b = *(reinterpret_cast<const uint4 *>(T + ci) + 1); /* hi[2..5], d7, first | count | biome */
        const uint32_t d = rt_dist(a, b, q);
        if (TIE ? d > s.best : d >= s.best) continue;
        const int cc = (int)((b.w >> 16) & 0xFFu);
        if (cc == 0) {
            if (!TIE || d < s.best) { s.best = d; s.res = ci; s.cnt = 1; }
            else if (s.cnt < 2) s.cnt++;
        } else {
            if constexpr (D == 0) return false;
            else if (!rt_walk<D - 1, TIE>(T, (int)(b.w & 0xFFFFu), cc, q, s)) return false;
        }
    }
    return true;
}
/* the same traversal as one loop with an explicit stack of (next child, end) per level: lanes of a warp
 * whose searches take different paths stay in step (one loop body), which the unrolled form, with one loop
 * per level, does not give when a warp's targets are unrelated (many seeds at scattered points) */
#define MG_RT_STACK 8
template <bool TIE>
static __device__ __noinline__ RtState rt_find_flat(const MgTreeNode *__restrict__ T, RtTarget q) {
    RtState s{0xFFFFFFFFu, -1, 0};
    int nxt[MG_RT_STACK], end[MG_RT_STACK];
    const uint32_t w = reinterpret_cast<const uint4 *>(T)[1].w;
    int sp = 0;
    nxt[0] = (int)(w & 0xFFFFu);
    end[0] = nxt[0] + (int)((w >> 16) & 0xFFu);
    while (sp >= 0) {
        const int ci = nxt[sp];
        if (ci >= end[sp]) { sp--; continue; }
        nxt[sp] = ci + 1;
        const uint4 a = *reinterpret_cast<const uint4 *>(T + ci);
        const uint4 b = *(reinterpret_cast<const uint4 *>(T + ci) + 1);
        const uint32_t d = rt_dist(a, b, q);
        if (TIE ? d > s.best : d >= s.best) continue;
        const int cc = (int)((b.w >> 16) & 0xFFu);
        if (cc == 0) {
            if (!TIE || d < s.best) { s.best = d; s.res = ci; s.cnt = 1; }
            else if (s.cnt < 2) s.cnt++;
        } else if (sp + 1 < MG_RT_STACK) {
            sp++;
            nxt[sp] = (int)(b.w & 0xFFFFu);
            end[sp] = nxt[sp] + cc;
        } else {
            s.res = -2; /* deeper than the stack: the 64-bit search decides */
            return s;
        }
    }
    return s;
}
template <bool TIE>
static __device__ __noinline__ RtState rt_find(const MgTreeNode *__restrict__ T, RtTarget q) {
    RtState s{0xFFFFFFFFu, -1, 0};
    const uint32_t w = reinterpret_cast<const uint4 *>(T)[1].w;
    if (!rt_walk<MG_RT_LEVELS, TIE>(T, (int)(w & 0xFFFFu), (int)((w >> 16) & 0xFFu), q, s)) s.res = -2;
    return s;
}
/* tree_search / tree_search_tie for warps whose cells are neighbours (grids, batches: similar targets, so
 * similar paths), tree_search_scattered for unrelated targets (many seeds, point lists, the seed search) */
__device__ __forceinline__ bool rt_packed(const MgTreeNode *__restrict__ T) {
    return (reinterpret_cast<const uint4 *>(T)[1].w >> 24) == MG_TREE_PACKED;
}
template <bool FLAT>
__device__ __forceinline__ int tree_search_t(const MgTreeNode *__restrict__ T, const int32_t *t, int cand, uint64_t &best) {
    RtTarget q;
    if (cand < 0 && rt_packed(T) && rt_target(t, q)) {
        const RtState s = FLAT ? rt_find_flat<false>(T, q) : rt_find<false>(T, q);
        if (s.res >= 0 && s.best < (uint32_t)MG_RT_CLAMP * MG_RT_CLAMP) {
            best = s.best;
            return s.res;
        }
    }
    return tree_search_stack(T, t, cand, best);
}
__device__ __forceinline__ int tree_search(const MgTreeNode *__restrict__ T, const int32_t *t, int cand, uint64_t &best) {
    return tree_search_t<false>(T, t, cand, best);
}
__device__ __forceinline__ int tree_search_scattered(const MgTreeNode *__restrict__ T, const int32_t *t, int cand,
                                                     uint64_t &best) {
    return tree_search_t<true>(T, t, cand, best);
}
__device__ __forceinline__ int tree_search_tie(const MgTreeNode *__restrict__ T, const int32_t *t, uint64_t &best,
                                               bool &tied) {
    RtTarget q;
    if (rt_packed(T) && rt_target(t, q)) {
        const RtState s = rt_find<true>(T, q);
        if (s.res >= 0 && s.best < (uint32_t)MG_RT_CLAMP * MG_RT_CLAMP) {
            best = s.best;
            tied = s.cnt >= 2;
            return s.res;
        }
    }
    return tree_search_tie_stack(T, t, best, tied);
}

/* ------------------------------------------------------------------ warp-shared R-tree candidates
 * The search's result is the first leaf in depth-first order at the minimum distance (a child is entered
 * iff its box is closer than the best leaf so far, a leaf replaces it iff strictly closer; every ancestor of
 * the first minimal leaf is at most as far, so the walk reaches it, and nothing after it is strictly closer).
 * So any list of leaves, in depth-first order, that holds every leaf able to be at the minimum for a target
 * gives the same leaf when scanned for the first strict minimum.  A warp's 32 cells are neighbours (an 8 x 4
 * block of a tile) with close targets: for the box B spanning them, a leaf whose distance to B (lower bound
 * over B) exceeds U, the least over leaves of their largest distance to a point of B, is farther than some
 * leaf for every target in B.  One walk per warp (the lanes take a node's children, up to 32 at once) lists
 * the leaves with lower bound <= U in depth-first order, U shrinking as leaves are met and starting from the
 * leaf a greedy descent reaches; each lane then scans only that list.  Both bounds use the packed 16-bit
 * distances with B's corners in place of the target (max(lo - Bhi, Blo - hi, 0) and max(lo - Blo, Bhi - hi,
 * 0) per dimension): a clamped lower bound is still a lower bound, and an upper bound is used only when
 * below MG_RT_CLAMP^2, where no dimension was clamped.  A list or stack that would overflow gives up (-1)
 * and the lanes search alone. */
#define MG_WC_CAND 128
#define MG_WC_STACK 128
/* the shared walk pays when a node's children fill most of a warp's lanes: trees built with 19 children per
 * node (26.3 on) take it; with 6 per node (26.1, 26.2) each step would use 6 of 32 lanes, and the lanes'
 * own level-unrolled searches measured faster */
#define MG_WARP_TREE_FANOUT 12
struct WarpTreeScratch {
    uint16_t cand[MG_WC_CAND];
    uint16_t stack[MG_WC_STACK];
};
__device__ __forceinline__ uint32_t rt_ub_or_inf(const uint4 &a, const uint4 &b, const RtTarget &ubq) {
    const uint32_t u = rt_dist(a, b, ubq);
    return u < (uint32_t)MG_RT_CLAMP * MG_RT_CLAMP ? u : 0xFFFFFFFFu;
}
/* all 32 lanes call it with the same box; returns the number of candidates in ws.cand, or -1 */
__device__ __forceinline__ int warp_tree_candidates(const MgTreeNode *__restrict__ T, const RtTarget &lbq,
                                                    const RtTarget &ubq, WarpTreeScratch &ws) {
    const unsigned FULL = 0xFFFFFFFFu;
    const int lane = threadIdx.x & 31;
    const uint32_t rw = reinterpret_cast<const uint4 *>(T)[1].w;
    /* greedy descent to a leaf (the child nearest to B at each level) for the first bound */
    uint32_t U = 0xFFFFFFFFu;
    {
        int first = (int)(rw & 0xFFFFu), count = (int)((rw >> 16) & 0xFFu);
        for (int depth = 0; depth < MG_RT_STACK; depth++) {
            if (count > 32) return -1; /* one lane per child */
            uint32_t lb = 0xFFFFFFFFu, w = 0;
            if (lane < count) {
                const uint4 a = *reinterpret_cast<const uint4 *>(T + first + lane);
                const uint4 b = *(reinterpret_cast<const uint4 *>(T + first + lane) + 1);
                lb = rt_dist(a, b, lbq);
                w = b.w;
            }
            const uint32_t m = __reduce_min_sync(FULL, lb);
            const int pick = __ffs(__ballot_sync(FULL, lb == m)) - 1;
            const uint32_t pw = __shfl_sync(FULL, w, pick);
            if (((pw >> 16) & 0xFFu) == 0) {
                const uint4 a = *reinterpret_cast<const uint4 *>(T + first + pick);
                const uint4 b = *(reinterpret_cast<const uint4 *>(T + first + pick) + 1);
                U = rt_ub_or_inf(a, b, ubq);
                break;
            }
            first = (int)(pw & 0xFFFFu);
            count = (int)((pw >> 16) & 0xFFu);
        }
    }
    /* depth-first walk; the stack holds pending nodes with the earliest in depth-first order on top */
    int sp = 1, nc = 0;
    if (lane == 0) ws.stack[0] = 0;
    __syncwarp();
    while (sp > 0) {
        const int node = ws.stack[--sp];
        const uint32_t nw = reinterpret_cast<const uint4 *>(T + node)[1].w;
        __syncwarp(); /* every lane has read the top before it is overwritten */
        const int count = (int)((nw >> 16) & 0xFFu);
        if (count == 0) { /* a leaf queued behind an internal sibling: it is next in depth-first order */
            if (nc >= MG_WC_CAND) return -1;
            if (lane == 0) ws.cand[nc] = (uint16_t)node;
            nc++;
            __syncwarp();
            continue;
        }
        if (count > 32) return -1;
        const int ci = (int)(nw & 0xFFFFu) + lane;
        bool keep = false, leaf = false;
        uint32_t ub = 0xFFFFFFFFu;
        if (lane < count) {
            const uint4 a = *reinterpret_cast<const uint4 *>(T + ci);
            const uint4 b = *(reinterpret_cast<const uint4 *>(T + ci) + 1);
            keep = rt_dist(a, b, lbq) <= U;
            leaf = ((b.w >> 16) & 0xFFu) == 0;
            if (keep && leaf) ub = rt_ub_or_inf(a, b, ubq);
        }
        U = min(U, __reduce_min_sync(FULL, ub));
        const unsigned km = __ballot_sync(FULL, keep);
        const unsigned im = __ballot_sync(FULL, keep && !leaf);
        /* leaves before the first internal survivor come next in depth-first order: listed now; the first
         * internal survivor and everything after it are pushed, the first on top */
        const unsigned em = im ? km & ((1u << (__ffs(im) - 1)) - 1u) : km;
        const unsigned pm = km & ~em;
        const unsigned lt = (1u << lane) - 1u;
        const int ne = __popc(em), np = __popc(pm);
        if (nc + ne > MG_WC_CAND || sp + np > MG_WC_STACK) return -1;
        if ((em >> lane) & 1u) ws.cand[nc + __popc(em & lt)] = (uint16_t)ci;
        if ((pm >> lane) & 1u) ws.stack[sp + np - 1 - __popc(pm & lt)] = (uint16_t)ci;
        nc += ne;
        sp += np;
        __syncwarp();
    }
    return nc;
}
/* first strict minimum of the packed distance over the listed leaves (the same for every lane's loop); with
 * TIE, also the leaves at that minimum, capped at 2 (the list holds every leaf that can be at the minimum, so
 * the count is the tree's) */
template <bool TIE = false>
__device__ __forceinline__ RtState rt_scan(const MgTreeNode *__restrict__ T, const uint16_t *cand, int n,
                                           const RtTarget &q) {
    RtState s{0xFFFFFFFFu, -1, 0};
    for (int k = 0; k < n; k++) {
        const int ci = cand[k];
        const uint4 a = *reinterpret_cast<const uint4 *>(T + ci);
        const uint4 b = *(reinterpret_cast<const uint4 *>(T + ci) + 1);
        const uint32_t d = rt_dist(a, b, q);
        if (d < s.best) { s.best = d; s.res = ci; s.cnt = 1; }
        else if (TIE && d == s.best && s.cnt < 2) s.cnt++;
    }
    return s;
}
/* tree_search (no candidate) for the 32 cells of a warp, called by all 32 lanes; lanes with active == false
 * take part in the walk and get -1.  Falls back to each lane's own search when the tree or a target is
 * outside the packed range or the list overflows, and to the 64-bit search when a lane's distance was
 * clamped. */
__device__ __forceinline__ int tree_search_warp(const MgTreeNode *__restrict__ T, const int32_t *t, bool active,
                                                WarpTreeScratch &ws) {
    const unsigned FULL = 0xFFFFFFFFu;
    RtTarget q{};
    const bool ok = !active || rt_target(t, q);
    const unsigned act = __ballot_sync(FULL, active);
    if (!act) return -1;
    int n = -1;
    if (rt_packed(T) && __all_sync(FULL, ok)) {
        int32_t lo[6], hi[6];
        for (int k = 0; k < 6; k++) {
            lo[k] = __reduce_min_sync(FULL, active ? t[k] : 0x7FFFFFFF);
            hi[k] = __reduce_max_sync(FULL, active ? t[k] : (int32_t)0x80000000);
        }
        RtTarget lbq, ubq;
        for (int k = 0; k < 3; k++) {
            lbq.p[k] = pack16(lo[2 * k], lo[2 * k + 1]);
            lbq.n[k] = pack16(-hi[2 * k], -hi[2 * k + 1]);
            ubq.p[k] = pack16(hi[2 * k], hi[2 * k + 1]);
            ubq.n[k] = pack16(-lo[2 * k], -lo[2 * k + 1]);
        }
        n = warp_tree_candidates(T, lbq, ubq, ws);
    }
    if (n >= 0) {
        const RtState s = rt_scan(T, ws.cand, n, q);
        __syncwarp(); /* the list is read by every lane before the warp's next walk */
        if (!active) return -1;
        if (s.res >= 0 && s.best < (uint32_t)MG_RT_CLAMP * MG_RT_CLAMP) return s.res;
        uint64_t d;
        return tree_search_stack(T, t, -1, d);
    }
    if (!active) return -1;
    uint64_t d;
    return tree_search(T, t, -1, d);
}
/* tree_search_tie for the 32 neighbouring cells of a warp (all lanes call it; inactive lanes get -1): the
 * first leaf at the minimum, its distance and whether a second leaf has the same distance */
__device__ __forceinline__ int tree_search_tie_warp(const MgTreeNode *__restrict__ T, const int32_t *t, bool active,
                                                    WarpTreeScratch &ws, uint64_t &best, bool &tied) {
    const unsigned FULL = 0xFFFFFFFFu;
    RtTarget q{};
    const bool ok = !active || rt_target(t, q);
    const unsigned act = __ballot_sync(FULL, active);
    if (!act) return -1;
    int n = -1;
    if (rt_packed(T) && __all_sync(FULL, ok)) {
        int32_t lo[6], hi[6];
        for (int k = 0; k < 6; k++) {
            lo[k] = __reduce_min_sync(FULL, active ? t[k] : 0x7FFFFFFF);
            hi[k] = __reduce_max_sync(FULL, active ? t[k] : (int32_t)0x80000000);
        }
        RtTarget lbq, ubq;
        for (int k = 0; k < 3; k++) {
            lbq.p[k] = pack16(lo[2 * k], lo[2 * k + 1]);
            lbq.n[k] = pack16(-hi[2 * k], -hi[2 * k + 1]);
            ubq.p[k] = pack16(hi[2 * k], hi[2 * k + 1]);
            ubq.n[k] = pack16(-lo[2 * k], -lo[2 * k + 1]);
        }
        n = warp_tree_candidates(T, lbq, ubq, ws);
    }
    if (n >= 0) {
        const RtState s = rt_scan<true>(T, ws.cand, n, q);
        __syncwarp();
        if (!active) return -1;
        if (s.res >= 0 && s.best < (uint32_t)MG_RT_CLAMP * MG_RT_CLAMP) {
            best = s.best;
            tied = s.cnt >= 2;
            return s.res;
        }
        return tree_search_tie_stack(T, t, best, tied);
    }
    if (!active) return -1;
    return tree_search_tie(T, t, best, tied);
}

/* (long)(v * 10000f) */
__device__ __forceinline__ int32_t quantize(float v) { return (int32_t)(int64_t)(v * 10000.0f); }

}  // namespace mgd
#endif
