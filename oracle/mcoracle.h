/* mcoracle.h -- CPU oracle for bit-exact multi-noise biome generation.
 *
 * TEST INFRASTRUCTURE ONLY.  Parity tests compare the GPU path with this library: tests/, the
 * smoke entry point and bench.py's CPU-baseline leg may load it; the product library
 * (libmcgen_gb300.so) never links, loads or calls it.
 *
 * It is a plain-C restatement of the reference engine's algorithm
 * (engine/mc_rng.h, mc_noise.h, mc_climate.h, mc_biomes.h, mc_end.h, mc_data.h)
 * plus libmcgen's biome-map semantics (libmcgen/src/region.c:61-122 zoom and
 * grid, libmcgen/src/biome.c:71-114 chunk-cell tie chain,
 * libmcgen/src/world.c:117-152 seed obfuscation).  Each function cites the
 * reference line range it follows.  Build with -ffp-contract=off and without
 * -ffast-math: the float/double operation order is part of the result.
 *
 * Parity is pinned against the reference's golden vectors
 * (tests/vectors/<V>/ climate, noise and grid-hash tables, tests/unit/ref26{2,3}.txt) and, in the build
 * container, against the reference engine compiled from its own sources
 * (oracle/build.py, build_reference).
 */
#ifndef MCORACLE_H
#define MCORACLE_H
#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* versions, dimensions, tie rules */
enum { OR_V26_1 = 0, OR_V26_2 = 1, OR_V26_3 = 2, OR_V26_4 = 3 };
enum { OR_OVERWORLD = 0, OR_NETHER = 1, OR_END = 2 };
/* How equal-fitness R-tree leaves are resolved:
 *   ENGINE     search without a candidate (engine/mc_biomes.h:58-62)
 *   GRID_CHAIN candidate = leaf of the previous cell, row-major iz outer
 *              (oracle/src/common/oracle/ClimateApi.java:35-58)
 *   CHUNK_CELL candidate chain along LevelChunkSection fill order
 *              (libmcgen/src/biome.c:71-114)                              */
enum { OR_TIE_ENGINE = 0, OR_TIE_GRID_CHAIN = 1, OR_TIE_CHUNK_CELL = 2 };

typedef struct OrWorld OrWorld;

/* Load one (version, dimension, preset) from a data root holding
 * data/climate-<V>.txt and data/params/<V>/{overworld,nether}.tsv.
 * preset: "normal"/"overworld", "amplified", "large_biomes" (Overworld only).
 * Returns NULL on error with a message in err. */
OrWorld *or_world_load(const char *root, const char *version, int dim, const char *preset,
                       char *err, size_t errlen);
void or_world_free(OrWorld *w);
int or_world_version(const OrWorld *w);
int or_world_float_mode(const OrWorld *w);
int or_tree_nodes(const OrWorld *w);
int or_tree_leaves(const OrWorld *w);

int or_biome_count(void);
const char *or_biome_name(int id);   /* without "minecraft:" */
int or_biome_id(const char *name);   /* accepts an optional "minecraft:" prefix */

/* BiomeManager.obfuscateSeed (libmcgen/src/world.c:117-152) */
int64_t or_hashed_seed(int64_t seed);

/* One NormalNoise value at noise-space coordinates (tests/vectors/<V>/noise.tsv
 * semantics).  which: 0 offset, 1 temperature, 2 vegetation, 3 continentalness,
 * 4 erosion, 5 ridge (Overworld world), 6 nether temperature, 7 nether
 * vegetation (Nether world).  Float-mode versions return the float widened. */
double or_noise_value(const OrWorld *w, int64_t seed, int which, double x, double y, double z);

/* Per-seed, per-point ENGINE-rule biomes (engine/cuda/mcg_host.c:36-83 semantics).
 * pts: 3 int32 quart coordinates per point.  out_biome[s*np+p]; out_tg (optional)
 * 6 int32 per sample (T,H,C,E,D,W; Nether T,H,0,0,0,0; End zeros).
 * threads <= 0 uses every core.  Parallel over seeds. */
void or_points(const OrWorld *w, const int64_t *seeds, int ns, const int32_t *pts, int np,
               uint8_t *out_biome, int32_t *out_tg, int threads);

/* Quart-resolution grid at one quart y: out[iz*nx+ix] for (qx0+ix, qy, qz0+iz).
 * rule: OR_TIE_ENGINE or OR_TIE_GRID_CHAIN (initial candidate: none).
 * Parallel over rows; the chain replay is sequential. */
void or_quart_grid(const OrWorld *w, int64_t seed, int qx0, int qz0, int nx, int nz, int qy,
                   int rule, uint8_t *out, int threads);

/* libmcgen drop-in semantics: BiomeManager zoom then the chunk-cell tie chain
 * (libmcgen/src/region.c:72-85, biome.c:87-114). */
int or_biome_at(const OrWorld *w, int64_t seed, int x, int y, int z);
/* mcgen_biome_grid: out[iz*nx+ix] = biome_at(x0+ix*step, y, z0+iz*step)
 * (libmcgen/src/region.c:86-122).  Parallel over rows. */
void or_biome_grid(const OrWorld *w, int64_t seed, int x0, int z0, int nx, int nz, int step, int y,
                   uint8_t *out, int threads);
/* 26.3 "chunk" mode grid (the Java oracle's chunk-batched climate): ties resolved by a candidate chain in
 * chunk order (chunk rows, then the chunk's cells z-major), across chunks.  Single-threaded: the chain is
 * sequential. */
void or_chunk_order_grid(const OrWorld *w, int64_t seed, int qx0, int qz0, int nx, int nz, int qy, uint8_t *out);
/* Quart grid with the chunk-cell tie chain per cell (no zoom). */
void or_chunk_grid(const OrWorld *w, int64_t seed, int qx0, int qz0, int nx, int nz, int qy, uint8_t *out, int threads);
/* mcgen_gpu_biome_points semantics: block points xyz[3n]. */
void or_block_points(const OrWorld *w, int64_t seed, int n, const int32_t *xyz, uint8_t *out, int threads);

/* Climate of one quart cell, as float (Overworld: T,H,C,E,D,W raw values;
 * Nether: T,H,0,0,0,0) and its quantised target; End: out[0] = erosion value. */
void or_cell_climate(const OrWorld *w, int64_t seed, int qx, int qy, int qz, float raw[6], int64_t tg[6]);
/* R-tree helpers on a quantised target: first minimum leaf (ENGINE), its
 * fitness, and the number of leaves at that fitness (capped at 2). */
int or_tree_find(const OrWorld *w, const int64_t tg[6], int64_t *dist, int *nmin);
/* Overworld density functions at block points: out[5 i + k], k = continents, erosion, ridges, offset, depth
 * (double branch: the doubles; float branch: the floats); -1 for other dimensions */
int or_density(const OrWorld *w, int64_t seed, int n, const int32_t *xyz, double *out);
int or_leaf_biome(const OrWorld *w, int leaf);
/* the R-tree as built (node bounds, links, biomes; child index array); returns the root */
int or_tree_export(const OrWorld *w, int64_t *lohi, int32_t *first_count_biome, int32_t *kids);
int or_tree_kids(const OrWorld *w);

/* Algorithmic work counters for one call of or_points on one seed: node-distance
 * evaluations in the R-tree search and octave samples, summed over the points.
 * Used to state the per-sample work that the roofline divides by. */
typedef struct { int64_t octave_samples, tree_nodes, tree_queries, spline_nodes; } OrWork;
void or_points_work(const OrWorld *w, int64_t seed, const int32_t *pts, int np, OrWork *work);

/* Biome seed search (crack/src/gpu_biomes/gpu_biomes.h:44-56 gb_search): every candidate seed of the
 * source is checked against the observations in order; reached[j] (nobs + 1 entries) counts the seeds
 * that passed exactly j leading observations; seeds passing all are returned sorted as unsigned, at most
 * max_found.  Sources: LIST (list[0..n)), STRUCTURE (base | i << 48, i < 65536), RANGE (base + i, i < n).
 * An observation is a quart cell (or, with OR_OBS_BLOCK, a block resolved through BiomeManager's zoom)
 * and a biome mask; flags' low byte is the End window half-width.  ties: also accept when any
 * minimum-fitness leaf's biome is in the mask. */
typedef struct { int32_t qx, qy, qz, flags; uint64_t mask[2]; } OrObs;
#define OR_OBS_BLOCK 0x100
enum { OR_SEEDS_LIST = 0, OR_SEEDS_STRUCTURE = 1, OR_SEEDS_RANGE = 2 };
void or_search(const OrWorld *w, int kind, const int64_t *list, uint64_t base, uint64_t n, const OrObs *obs, int nobs,
               int ties, uint64_t *reached, int64_t *found, uint32_t max_found, uint32_t *n_found, int threads);
int or_obs_end_radius(const OrWorld *w, const uint64_t mask[2]);

/* FNV-1a 64 over "minecraft:<name>\n" per cell (biome_grid_hashes.tsv digest). */
uint64_t or_fnv1a64_names(const uint8_t *ids, size_t n);

#ifdef __cplusplus
}
#endif
#endif
