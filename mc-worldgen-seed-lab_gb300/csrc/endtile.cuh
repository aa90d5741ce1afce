/* endtile.cuh -- End island classes of an 8 x 8-chunk tile, shared by the batched kernel and the plain
 * per-request End path.
 *
 * TheEndBiomeSource's class of chunk c needs the island field at the 25 x 25 chunk cells around c
 * (engine/mc_end.h:66-119).  A tile evaluates the simplex field once over its 32 x 32-cell window -- one
 * window row per warp, kept as 32-bit island masks -- instead of 625 times per chunk; then two lanes per
 * chunk visit only the island bits of their half of the 25 window rows (the maximum does not depend on the
 * order).  Needs a 128-thread block. */
#ifndef MG_ENDTILE_CUH
#define MG_ENDTILE_CUH
#include "climate.cuh"

namespace mg {

#define END_TC 8       /* chunks per End tile side */
#define END_WIN (END_TC + 24)

struct EndTile {
    uint32_t rows[END_WIN];            /* bit i of rows[r]: window cell (i, r) is an island */
    float isize[END_WIN * END_WIN];    /* its size */
    uint8_t cls[END_TC * END_TC];      /* class of tile chunk (cx0 + i % 8, cz0 + i / 8) */
};
static_assert(END_WIN == 32 && END_TC * END_TC * 2 == 128, "End tile layout: a warp fills one window row");

/* classes of chunks [cx0, cx0 + 8) x [cz0, cz0 + 8) into e.cls; p: the End simplex permutation */
template <bool FM>
__device__ __forceinline__ void end_tile_classes(const uint8_t *__restrict__ p, double F2, double G2, int cx0, int cz0,
                                                 EndTile &e) {
    /* chunk c's height reads chunk cells c' + d, d in [-12, 12], with c' = (2c+1)/2 in Java int division
     * (c for c >= 0, c + 1 for c < 0): a window of at most END_TC - 1 + 25 cells per axis */
    const int wx0 = (cx0 * 2 + 1) / 2 - 12, wz0 = (cz0 * 2 + 1) / 2 - 12;
    for (int i = threadIdx.x; i < END_WIN * END_WIN; i += blockDim.x) { /* 8 rounds, a window row per warp */
        const long long tx = (long long)wx0 + i % END_WIN, tz = (long long)wz0 + i / END_WIN;
        bool isl = false;
        float size = 0.0f;
        if (tx * tx + tz * tz > 4096LL) {
            isl = end_island(p, (double)tx, (double)tz, F2, G2, FM);
            if (isl) size = fmodf(fabsf((float)tx) * 3439.0f + fabsf((float)tz) * 147.0f, 13.0f) + 9.0f;
        }
        e.isize[i] = size;
        const uint32_t m = __ballot_sync(0xFFFFFFFFu, isl);
        if ((threadIdx.x & 31) == 0) e.rows[i >> 5] = m;
    }
    __syncthreads();
    /* two threads per chunk, each over half of the 25 window rows, visiting only the rows' island bits; the
     * maximum does not depend on the order */
    {
        const int c = threadIdx.x >> 1, half = threadIdx.x & 1;
        const int cx = cx0 + c % END_TC, cz = cz0 + c / END_TC;
        const bool outer = (long long)cx * cx + (long long)cz * cz > 4096LL;
        const int bx = (cx * 2 + 1) * 8, bz = (cz * 2 + 1) * 8;
        float best = -100.0f;
        if (outer) {
            const int sx = bx / 8, sz = bz / 8;
            const int ccx = sx / 2, ccz = sz / 2, ox = sx % 2, oz = sz % 2;
            if (!FM) {
                int32_t sq = (int32_t)((uint32_t)sx * (uint32_t)sx + (uint32_t)sz * (uint32_t)sz);
                float len = (float)sqrt((double)(float)sq);
                best = clampf(100.0f - len * 8.0f, -100.0f, 80.0f);
            }
            const int sh = ccx - 12 - wx0; /* 0 .. END_TC - 1 */
            for (int dz = half ? 1 : -12; dz <= (half ? 12 : 0); dz++) {
                const int row = ccz + dz - wz0;
                uint32_t m = (e.rows[row] >> sh) & 0x1FFFFFFu;
                while (m) {
                    const int b = __ffs((int)m) - 1;
                    m &= m - 1;
                    const int dx = b - 12;
                    const float xd = (float)(ox - dx * 2), zd = (float)(oz - dz * 2);
                    const float h = clampf(100.0f - (float)sqrt((double)(xd * xd + zd * zd)) * e.isize[row * END_WIN + b + sh], -100.0f, 80.0f);
                    best = best > h ? best : h;
                }
            }
        }
        const float other = __shfl_xor_sync(0xFFFFFFFFu, best, 1);
        best = best > other ? best : other;
        if (half == 0) {
            int cls = 0;
            if (outer) {
                double ev;
                if (!FM) ev = ((double)best - 8.0) / 128.0;
                else {
                    const float ddx = (float)(0 - bx), ddz = (float)(0 - bz);
                    const float len = (float)sqrt((double)(ddx * ddx + 0.0f * 0.0f + ddz * ddz));
                    const float cc = (clampf(100.0f - len, -100.0f, 80.0f) - 8.0f) * 0.0078125f;
                    const float o = (best - 8.0f) / 128.0f;
                    ev = (double)(cc > o ? cc : o);
                }
                cls = ev > 0.25 ? 1 : (ev >= -0.0625 ? 2 : (ev < -0.21875 ? 3 : 4));
            }
            e.cls[c] = (uint8_t)cls;
        }
    }
    __syncthreads();
}

}  // namespace mg
#endif
