/* search.cuh -- device pieces of the biome seed search (crack/src/gpu_biomes/gpu_biomes.cu k_search,
 * engine/cuda/mc_gpu.cuh:47-194): per-candidate BiomeManager seed (SHA-256), observation cells, biome
 * masks and the equal-fitness leaf set used by the ties mode. */
#ifndef MG_SEARCH_CUH
#define MG_SEARCH_CUH

#include "climate.cuh"

namespace mg {

/* FIPS 180-4 round constants */
static __constant__ uint32_t kSha256K[64] = {
    0x428a2f98, 0x71374491, 0xb5c0fbcf, 0xe9b5dba5, 0x3956c25b, 0x59f111f1, 0x923f82a4, 0xab1c5ed5,
    0xd807aa98, 0x12835b01, 0x243185be, 0x550c7dc3, 0x72be5d74, 0x80deb1fe, 0x9bdc06a7, 0xc19bf174,
    0xe49b69c1, 0xefbe4786, 0x0fc19dc6, 0x240ca1cc, 0x2de92c6f, 0x4a7484aa, 0x5cb0a9dc, 0x76f988da,
    0x983e5152, 0xa831c66d, 0xb00327c8, 0xbf597fc7, 0xc6e00bf3, 0xd5a79147, 0x06ca6351, 0x14292967,
    0x27b70a85, 0x2e1b2138, 0x4d2c6dfc, 0x53380d13, 0x650a7354, 0x766a0abb, 0x81c2c92e, 0x92722c85,
    0xa2bfe8a1, 0xa81a664b, 0xc24b8b70, 0xc76c51a3, 0xd192e819, 0xd6990624, 0xf40e3585, 0x106aa070,
    0x19a4c116, 0x1e376c08, 0x2748774c, 0x34b0bcb5, 0x391c0cb3, 0x4ed8aa4a, 0x5b9cca4f, 0x682e6ff3,
    0x748f82ee, 0x78a5636f, 0x84c87814, 0x8cc70208, 0x90befffa, 0xa4506ceb, 0xbef9a3f7, 0xc67178f2};

__device__ __forceinline__ uint32_t ror32(uint32_t x, int n) { return __funnelshift_r(x, x, n); }

/* BiomeManager.obfuscateSeed: the first 8 bytes of SHA-256 over the seed's 8 little-endian bytes, read as
 * a little-endian long (libmcgen/src/world.c:117-152).  One 64-byte block; the message schedule is kept
 * as a 16-word ring. */
__device__ __forceinline__ int64_t hashed_seed(int64_t seed) {
    const uint64_t u = (uint64_t)seed;
    uint32_t w[16];
    w[0] = __byte_perm((uint32_t)u, 0, 0x0123);
    w[1] = __byte_perm((uint32_t)(u >> 32), 0, 0x0123);
    w[2] = 0x80000000u;
#pragma unroll
    for (int i = 3; i < 15; i++) w[i] = 0;
    w[15] = 64;
    uint32_t a = 0x6a09e667, b = 0xbb67ae85, c = 0x3c6ef372, d = 0xa54ff53a;
    uint32_t e = 0x510e527f, f = 0x9b05688c, g = 0x1f83d9ab, h = 0x5be0cd19;
#pragma unroll
    for (int i = 0; i < 64; i++) {
        uint32_t wi;
        if (i < 16) {
            wi = w[i];
        } else {
            const uint32_t w15 = w[(i - 15) & 15], w2 = w[(i - 2) & 15];
            wi = w[i & 15] + (ror32(w15, 7) ^ ror32(w15, 18) ^ (w15 >> 3)) + w[(i - 7) & 15] +
                 (ror32(w2, 17) ^ ror32(w2, 19) ^ (w2 >> 10));
            w[i & 15] = wi;
        }
        const uint32_t t1 = h + (ror32(e, 6) ^ ror32(e, 11) ^ ror32(e, 25)) + ((e & f) ^ (~e & g)) + kSha256K[i] + wi;
        const uint32_t t2 = (ror32(a, 2) ^ ror32(a, 13) ^ ror32(a, 22)) + ((a & b) ^ (a & c) ^ (b & c));
        h = g; g = f; f = e; e = d + t1;
        d = c; c = b; b = a; a = t1 + t2;
    }
    const uint32_t h0 = 0x6a09e667u + a, h1 = 0xbb67ae85u + b;
    /* digest bytes 0..7 are h0, h1 big-endian; as a little-endian long */
    return (int64_t)(((uint64_t)__byte_perm(h1, 0, 0x0123) << 32) | __byte_perm(h0, 0, 0x0123));
}

__device__ __forceinline__ bool obs_in(const MgObs &o, int b) { return (o.mask[b >> 6] >> (b & 63)) & 1ULL; }

/* the observation's quart cell for this seed (engine/cuda/mc_gpu.cuh:120-124); the hashed seed is
 * formed once per seed, at the first block observation */
__device__ __forceinline__ void obs_cell(const MgObs &o, int64_t seed, int64_t &hs, bool &have, int &qx, int &qy, int &qz) {
    if (!(o.flags & MG_OBS_BLOCK)) { qx = o.qx; qy = o.qy; qz = o.qz; return; }
    if (!have) { hs = hashed_seed(seed); have = true; }
    zoom_cell(hs, o.qx, o.qy, o.qz, qx, qy, qz);
}

/* biomes of every leaf at the minimum fitness (engine/cuda/mc_gpu.cuh:166-187): a child is visited iff its
 * box distance is <= the best leaf distance so far; a closer leaf resets the set */
__device__ __forceinline__ void tree_ties(const MgTreeNode *__restrict__ T, const int32_t *t, uint64_t m[2]) {
    int stk_node[10], stk_next[10], sp = 1;
    uint64_t best = ~0ULL;
    m[0] = m[1] = 0;
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
            if (cd < best) { best = cd; m[0] = m[1] = 0; }
            const int b = T[ci].biome;
            m[b >> 6] |= 1ULL << (b & 63);
        } else if (sp < 10) {
            stk_node[sp] = ci; stk_next[sp] = 0; sp++;
        }
    }
}

/* observation met by a target: its ENGINE biome is in the mask, or (ties) any equal-fitness leaf's is.  The
 * ENGINE leaf is one of the equal-fitness leaves, so in ties mode the one traversal that collects their
 * biomes decides alone. */
__device__ __forceinline__ bool obs_accept(const MgObs &o, const MgTreeNode *__restrict__ T, const int32_t *tg, bool ties) {
    if (!ties) {
        uint64_t d;
        return obs_in(o, T[tree_search_scattered(T, tg, -1, d)].biome);
    }
    uint64_t m[2];
    tree_ties(T, tg, m);
    return ((m[0] & o.mask[0]) | (m[1] & o.mask[1])) != 0;
}

/* The End check of an observation, deciding early (same answer as the full window).
 * The class of a chunk is a step function of the highest island height h in its window, and h only grows
 * as islands are visited, so the class only moves up the order small islands < barrens < midlands <
 * highlands.  The window's cells are visited nearest first; the visit stops when (a) every class still
 * reachable is in the mask (accept) or none is (reject), or (b) no remaining cell can raise h: a cell at
 * offset (dx, dz) gives at most 100 - 9 sqrt(lb) with lb <= |offset|^2 (island size >= 9). */
struct EndOrder {
    int8_t dx[625], dz[625];
    uint16_t lb[625]; /* ((2|dx| - 1)+)^2 + ((2|dz| - 1)+)^2, a lower bound of xd^2 + zd^2 */
};
constexpr EndOrder make_end_order() {
    EndOrder t{};
    int n = 0;
    for (int dx = -12; dx <= 12; dx++)
        for (int dz = -12; dz <= 12; dz++) {
            const int ax = dx < 0 ? -dx : dx, az = dz < 0 ? -dz : dz;
            const int bx = 2 * ax - 1 > 0 ? 2 * ax - 1 : 0, bz = 2 * az - 1 > 0 ? 2 * az - 1 : 0;
            t.dx[n] = (int8_t)dx;
            t.dz[n] = (int8_t)dz;
            t.lb[n] = (uint16_t)(bx * bx + bz * bz);
            n++;
        }
    for (int i = 1; i < 625; i++) /* insertion sort by lb (stable) */
        for (int j = i; j > 0 && t.lb[j - 1] > t.lb[j]; j--) {
            const int8_t a = t.dx[j], b = t.dz[j];
            const uint16_t c = t.lb[j];
            t.dx[j] = t.dx[j - 1]; t.dz[j] = t.dz[j - 1]; t.lb[j] = t.lb[j - 1];
            t.dx[j - 1] = a; t.dz[j - 1] = b; t.lb[j - 1] = c;
        }
    return t;
}
static __constant__ EndOrder kEndOrder = make_end_order();

/* class rank 0..3 (small islands, barrens, midlands, highlands) of a chunk outside the central disc */
__device__ __forceinline__ int end_rank(double e) {
    return e > 0.25 ? 3 : (e >= -0.0625 ? 2 : (e < -0.21875 ? 0 : 1));
}
template <bool FM>
__device__ __forceinline__ bool end_accept(const MgWorldDesc &W, const uint8_t *__restrict__ p, const MgObs &o, int qx,
                                           int qz) {
    const int cx = (qx * 4) >> 4, cz = (qz * 4) >> 4;
    if ((long long)cx * cx + (long long)cz * cz <= 4096LL) return obs_in(o, W.end_ids[0]);
    const int rad = o.flags & 0xFF;
    /* rank k -> class id: small islands, barrens, midlands, highlands */
    const int cls_of_rank[4] = {W.end_ids[3], W.end_ids[4], W.end_ids[2], W.end_ids[1]};
    bool in[4];
    for (int k = 0; k < 4; k++) in[k] = obs_in(o, cls_of_rank[k]);
    const int bx = (cx * 2 + 1) * 8, bz = (cz * 2 + 1) * 8;
    const int sx = bx / 8, sz = bz / 8;
    const int ccx = sx / 2, ccz = sz / 2, ox = sx % 2, oz = sz % 2;
    float best;
    float cdist = 0.0f;
    if (!FM) {
        int32_t sq = (int32_t)((uint32_t)sx * (uint32_t)sx + (uint32_t)sz * (uint32_t)sz);
        float len = (float)sqrt((double)(float)sq);
        best = clampf(100.0f - len * 8.0f, -100.0f, 80.0f);
    } else {
        best = -100.0f;
        const float ddx = (float)(0 - bx), ddz = (float)(0 - bz);
        const float len = (float)sqrt((double)(ddx * ddx + 0.0f * 0.0f + ddz * ddz));
        cdist = (clampf(100.0f - len, -100.0f, 80.0f) - 8.0f) * 0.0078125f;
    }
    auto rank_now = [&]() {
        if (!FM) return end_rank(((double)best - 8.0) / 128.0);
        const float o2 = (best - 8.0f) / 128.0f;
        return end_rank((double)(cdist > o2 ? cdist : o2));
    };
    for (int i = 0; i < 625; i++) {
        int r = rank_now();
        bool any = false, all = true;
        for (int k = r; k < 4; k++) { any |= in[k]; all &= in[k]; }
        if (all) return true;
        if (!any) return false;
        const int lb = kEndOrder.lb[i];
        if (100.0f - 9.0f * sqrtf((float)lb) <= best) break; /* nothing left can raise h */
        const int dx = kEndOrder.dx[i], dz = kEndOrder.dz[i];
        if (dx < -rad || dx > rad || dz < -rad || dz > rad) continue;
        const long long tx = (long long)ccx + dx, tz = (long long)ccz + dz;
        if (tx * tx + tz * tz <= 4096LL) continue;
        if (!end_island(p, (double)tx, (double)tz, W.end_f2, W.end_g2, FM)) continue;
        const float size = fmodf(fabsf((float)tx) * 3439.0f + fabsf((float)tz) * 147.0f, 13.0f) + 9.0f;
        const float xd = (float)(ox - dx * 2), zd = (float)(oz - dz * 2);
        const float h = clampf(100.0f - (float)sqrt((double)(xd * xd + zd * zd)) * size, -100.0f, 80.0f);
        best = best > h ? best : h;
    }
    return in[rank_now()];
}

/* candidate i of a source: 0 list, 1 structure seed base | i << 48, 2 base + i */
__device__ __forceinline__ int64_t search_seed(int kind, const int64_t *__restrict__ list, uint64_t base, uint64_t i) {
    if (kind == 0) return list[i];
    if (kind == 1) return (int64_t)(base | (i << 48));
    return (int64_t)(base + i);
}

}  // namespace mg
#endif
