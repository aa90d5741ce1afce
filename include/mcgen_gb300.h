/* mcgen_gb300.h -- additions to the libmcgen ABI (include/mcgen.h) for the GB300 biome engine.
 *
 * New symbols only; nothing in mcgen.h changes meaning.  They expose the forms the reference serves
 * through other entry points:
 *  - many seeds x fixed quart points, ENGINE tie rule: the reference engine's batch API
 *    (crack/src/gpu_biomes/gpu_biomes.h:22-57 gb_points_gpu; CPU twin engine/cuda/mcg_host.c:36-83
 *    mcg_ref_points);
 *  - quart-resolution grids with an explicit tie rule: the reference's golden grids
 *    (oracle/src/common/oracle/ClimateApi.java:35-58, GRID_CHAIN) and the engine's point queries
 *    (engine/mc_biomes.h:58-62, ENGINE);
 *  - device-pointer variants of the above and of mcgen_biome_grid, taking a cudaStream_t as void*, for
 *    callers whose inputs already live in GPU memory.
 *
 * Tie rules (about 0.04% of Overworld cells have two R-tree leaves at equal fitness):
 *   MCGEN_TIE_ENGINE     first minimum leaf in tree order (search without a candidate);
 *   MCGEN_TIE_GRID_CHAIN candidate = leaf of the previous cell, row-major (iz outer);
 *   MCGEN_TIE_CHUNK_CELL candidate chain along the chunk's fill order (what mcgen_biome_grid uses);
 *   MCGEN_TIE_CHUNK_ORDER candidate chain chunk by chunk (chunk rows, then each chunk's cells z-major) across
 *                        the grid: 26.3's chunk-batched climate, the reference Java oracle's "chunk" mode
 *                        (oracle/src/v263/oracle/compat/Compat.java:168-221) that its `chunk` golden digests pin.
 */
#ifndef MCGEN_GB300_H
#define MCGEN_GB300_H
#include "mcgen.h"
#ifdef __cplusplus
extern "C" {
#endif

enum { MCGEN_TIE_ENGINE = 0, MCGEN_TIE_GRID_CHAIN = 1, MCGEN_TIE_CHUNK_CELL = 2, MCGEN_TIE_CHUNK_ORDER = 3 };

/* Version / dimension / preset / seed of a world (McWorld is opaque in mcgen.h). */
MCGEN_API int mcgen_gb300_world_info(const McWorld *w, int *version, int *dimension, int64_t *climate_seed,
                                     int *float_branch);

/* Quart grid at quart y for the world's climate seed: out[iz*nx+ix] = biome of quart cell
 * (qx0+ix, qy, qz0+iz), no zoom.  tie_rule: MCGEN_TIE_ENGINE, MCGEN_TIE_GRID_CHAIN or
 * MCGEN_TIE_CHUNK_ORDER (the initial candidate is none).  New in this library; the reference computes these grids in its Java oracle
 * (ClimateApi.grid) and, per point, in engine/cuda/mcg_host.c:36-83. */
MCGEN_API int mcgen_gb300_quart_grid(const McWorld *w, int qx0, int qz0, int nx, int nz, int qy, int tie_rule,
                                     uint8_t *out);

/* Many seeds x fixed quart points, ENGINE rule: out[s*np+p] for seeds[s] at quart point
 * qxyz[3p..3p+2]; targets (optional) receives the 6 quantised climate values per sample
 * (Nether T,H,0,0,0,0; End zeros).  The world supplies version, dimension and preset; its own seed is
 * ignored.  Replaces crack/src/gpu_biomes/gpu_biomes.h:22-57 gb_points_gpu (host buffers). */
MCGEN_API int mcgen_gb300_seed_points(const McWorld *w, const int64_t *seeds, int ns, const int32_t *qxyz, int np,
                                      uint8_t *out, int32_t *targets);

/* Overworld density functions at block points for `seed` (the world supplies version and preset):
 * out[5i + k] for point xyz[3i..3i+2] = continents, erosion, ridges, offset, depth -- the values the climate
 * sampler computes before it rounds them to floats for the biome search (double branch 26.1/26.2: the exact
 * doubles; float branch: the floats, widened).  The reference computes them in its Java oracle ("df",
 * oracle/gen_vectors.py:76-84; tests/vectors/<V>/df.tsv) and inside engine/mc_climate.h:113-164 at block
 * coordinates.  MCGEN_E_ARG for Nether and End worlds. */
MCGEN_API int mcgen_gb300_density_values(const McWorld *w, int64_t seed, int n, const int32_t *xyz, double *out);

/* Device-pointer forms: every pointer is CUDA device memory, work is queued on `stream`
 * (a cudaStream_t, NULL = the legacy default stream) and the call returns without synchronising. */
MCGEN_API int mcgen_gb300_seed_points_dev(const McWorld *w, const int64_t *d_seeds, int ns, const int32_t *d_qxyz,
                                          int np, uint8_t *d_out, int32_t *d_targets, void *stream);
MCGEN_API int mcgen_gb300_biome_grid_dev(const McWorld *w, int x0, int z0, int nx, int nz, int step, int y,
                                         uint8_t *d_out, void *stream);
MCGEN_API int mcgen_gb300_quart_grid_dev(const McWorld *w, int qx0, int qz0, int nx, int nz, int qy, int tie_rule,
                                         uint8_t *d_out, void *stream);

/* One quart grid for an explicit seed (the world supplies version, dimension and preset), device output:
 * the plain per-request form -- one setup launch and one grid launch per call. */
MCGEN_API int mcgen_gb300_quart_grid_seed_dev(const McWorld *w, int64_t seed, int qx0, int qz0, int nx, int nz,
                                              int qy, int tie_rule, uint8_t *d_out, void *stream);

/* ---- batched form: many biome-map requests of uneven size in one persistent launch ----
 * A request is a quart-resolution region (qx0.., qz0.., nx x nz at quart y) of one world (version,
 * dimension, preset) and seed.  A plan freezes a request list: it builds every distinct (world, seed)'s
 * noise lattices into a pool, splits requests into tiles that one persistent kernel takes from a device
 * work queue, and lays outputs back to back (request i's nx*nz ids, row-major, at output offset i).
 * Runs replay a CUDA graph of the setup and batch launches.  tie_rule: MCGEN_TIE_ENGINE or
 * MCGEN_TIE_CHUNK_CELL (each cell resolved as the chunk that holds it stores it). */
typedef struct McGb300Request {
    const McWorld *world; /* version, dimension, preset; its own seed is ignored */
    int64_t seed;
    int32_t qx0, qz0, nx, nz, qy;
} McGb300Request;
typedef struct McGb300Plan McGb300Plan;
/* A plan keeps each of its worlds alive until mcgen_gb300_plan_free: mcgen_world_free on such a world only
 * marks it, and the plan's free releases it (the plan reads the world's description and device tree). */
MCGEN_API int mcgen_gb300_plan_new(const McGb300Request *reqs, int n, int tie_rule, McGb300Plan **out);
MCGEN_API void mcgen_gb300_plan_free(McGb300Plan *p);
MCGEN_API long long mcgen_gb300_plan_output_bytes(const McGb300Plan *p);
MCGEN_API long long mcgen_gb300_plan_output_offset(const McGb300Plan *p, int i);
/* the tile shape in use (cells x rows, resident CTAs per SM): 0 (8 x 16, 9), 1 (8 x 16, 7), 2 (8 x 16, 6),
 * 3 (8 x 16, 8) */
MCGEN_API int mcgen_gb300_plan_shape(const McGb300Plan *p);
MCGEN_API int mcgen_gb300_plan_set_shape(McGb300Plan *p, int shape);
/* bytes plan_new copied to the device (worlds, request and setup lists) */
MCGEN_API long long mcgen_gb300_plan_h2d_bytes(const McGb300Plan *p);
/* time the four tile shapes on this plan (reps runs each into d_out) and keep the fastest */
MCGEN_API int mcgen_gb300_plan_autotune(McGb300Plan *p, uint8_t *d_out, int reps, double *best_ms);
/* run into device memory on `stream` (graph replay) / without a graph / into host memory (direct launches,
 * outputs copied back, synchronous).  Runs of one plan share its lattice pool and tile counter, so each run
 * is ordered after the plan's previous run on the GPU (the library makes `stream` wait for it); runs of
 * different plans are independent.  mcgen_gb300_plan_free does not block: the plan's device memory returns
 * to the library's pool after its last run. */
MCGEN_API int mcgen_gb300_plan_run_dev(McGb300Plan *p, uint8_t *d_out, void *stream);
MCGEN_API int mcgen_gb300_plan_run_dev_direct(McGb300Plan *p, uint8_t *d_out, void *stream);
MCGEN_API int mcgen_gb300_plan_run(McGb300Plan *p, uint8_t *out);

/* ---- served form: continuous batching with a device noise-state cache ----
 * Submit requests from any thread at any time; a worker admits every pending request into the next batch
 * as soon as one of `max_inflight` streams is free, so requests that arrive while others run are batched
 * and overlap with them on the GPU.  Each (world, seed)'s lattices stay resident in an HBM cache of
 * `hbm_budget_bytes` (LRU among entries no running batch uses).  `out` receives nx*nz ids (row-major) and
 * must stay valid until mcgen_gb300_server_wait returns for the ticket.  Results equal the batched and
 * plain forms bit for bit (ENGINE tie rule). */
typedef struct McGb300Server McGb300Server;
typedef struct McGb300ServerStats {
    long long requests_submitted, requests_admitted, batches, samples_done;
    long long cache_hits, cache_misses, cache_evictions, cache_entries, pending;
    long long cache_slots[3]; /* Overworld, Nether, End */
} McGb300ServerStats;
MCGEN_API int mcgen_gb300_server_new(long long hbm_budget_bytes, int max_inflight, int max_batch_requests,
                                     McGb300Server **out);
MCGEN_API void mcgen_gb300_server_free(McGb300Server *s); /* drains pending work first */
MCGEN_API int mcgen_gb300_server_submit(McGb300Server *s, const McGb300Request *req, uint8_t *out, long long *ticket);
/* wait for a ticket (timeout_ms < 0: no limit; MCGEN_E_CANCEL on timeout, the ticket stays valid);
 * latency_ms: submit to completion.  A ticket can be waited for once.
 * Errors: a batch that fails while forming (allocation, copy, launch) fails its requests with that error and
 * leaves no partly built noise state in the cache; after an allocation failure (MCGEN_E_NOMEM) the server
 * goes on serving, after any other error every pending and later request fails with it.  A submitted
 * request keeps its world alive until it completes (mcgen_world_free meanwhile only marks the world). */
MCGEN_API int mcgen_gb300_server_wait(McGb300Server *s, long long ticket, int timeout_ms, double *latency_ms);
MCGEN_API int mcgen_gb300_server_stats(McGb300Server *s, McGb300ServerStats *out);
/* Measurement hook (a load generator for the served form): replay an open-loop arrival schedule -- request i
 * submitted by a native thread at arrival_s[i] seconds after the call starts, its ids into out + out_off[i]
 * -- and wait for every ticket; latency_ms[i] runs from the scheduled arrival to completion (a submitter
 * behind schedule adds to it).  *elapsed_s: the whole replay.  The first error is returned. */
MCGEN_API int mcgen_gb300_server_replay(McGb300Server *s, const McGb300Request *reqs, const double *arrival_s, int n,
                                        uint8_t *out, const long long *out_off, double *latency_ms, double *elapsed_s);
/* Testing aid: the next batch the server forms fails at its device-allocation step with `code` (> 0), as if
 * that allocation had failed; host-side only, no device fault. */
MCGEN_API int mcgen_gb300_server_fail_next(McGb300Server *s, int code);

/* ---- biome seed search: which candidate seeds produce the observed biomes ----
 * The reference's gb_search (crack/src/gpu_biomes/gpu_biomes.h:44-56, gpu_biomes.cu:245-278).  Candidates:
 * MCGEN_SEEDS_LIST list[0..n), MCGEN_SEEDS_STRUCTURE base | i << 48 for i < 65536 (base: a 48-bit structure
 * seed; n ignored), MCGEN_SEEDS_RANGE base + i for i < n.  Each candidate is checked against obs[0..nobs)
 * in order and stops at the first observation it fails; reached[j] (nobs + 1 entries) counts candidates
 * that passed exactly j observations.  Candidates passing all are written to found, sorted as unsigned, at
 * most max_found (*n_found of them; when more pass, which ones is unspecified, as in the reference).  An observation (the reference's McgObs, engine/cuda/mc_gpu.cuh:47-54)
 * is a quart cell, or with MCGEN_OBS_BLOCK in flags a block that BiomeManager's zoom resolves with the
 * candidate's hashed seed, and the set of biome ids that satisfy it (mask bit id); flags' low byte is the
 * End window half-width (12 in the game; mcgen_gb300_obs_end_radius gives the narrowest exact one).
 * ties != 0: an Overworld/Nether observation is also met when any equal-fitness R-tree leaf's biome is in
 * the mask (the game's choice between them is not deterministic).  *ms: device time of the search. */
typedef struct McGb300Obs {
    int32_t qx, qy, qz, flags;
    uint64_t mask[2];
} McGb300Obs;
#define MCGEN_OBS_BLOCK 0x100
enum { MCGEN_SEEDS_LIST = 0, MCGEN_SEEDS_STRUCTURE = 1, MCGEN_SEEDS_RANGE = 2 };
MCGEN_API int mcgen_gb300_search(const McWorld *w, int kind, const int64_t *list, uint64_t base, uint64_t n,
                                 const McGb300Obs *obs, int nobs, int ties, int64_t *found, uint32_t max_found,
                                 uint32_t *n_found, uint64_t *reached, double *ms);
/* End window half-width for an observation mask (engine/cuda/mc_gpu.cuh:640-652); -1 on bad arguments */
MCGEN_API int mcgen_gb300_obs_end_radius(const McWorld *w, const uint64_t mask[2]);

/* Allocation-free form of mcgen_gb300_seed_points_dev, for callers that cannot let a library allocate
 * device memory (their own memory arena, latency-critical loops, no allocation after set-up).  No
 * counterpart in the reference.  The per-seed noise lattices go to one fixed 16 MiB device array inside
 * the library instead of per-call scratch, so ns * (lattices per seed) * 352 bytes must fit: at most 1,036
 * Overworld, 5,957 Nether or 47,662 End seeds per call; larger calls return MCGEN_E_ARG (split them).
 * The caller passes device inputs and outputs as for _dev.  The world must already be on the device (any
 * earlier biome call on it puts it there), else MCGEN_E_ARG.  The first call on a device looks up the
 * array's address; make it before any stream capture.  Calls share the array: calls whose GPU work
 * overlaps race on it. */
MCGEN_API int mcgen_gb300_seed_points_noalloc(const McWorld *w, const int64_t *d_seeds, int ns, const int32_t *d_qxyz,
                                              int np, uint8_t *d_out, int32_t *d_targets, void *stream);

/* Number of kernel launches the library issued since load (for launch accounting in benchmarks). */
MCGEN_API long long mcgen_gb300_launch_count(void);

/* Per-kernel timing of the library's own launches: while enabled, each launch is bracketed by two CUDA
 * events on its stream.  mcgen_gb300_profile(1) clears and starts, (0) stops; profile_read returns kernel
 * `kernel`'s name (k_setup_xo, k_points, ...), summed milliseconds and launch count; MCGEN_E_ARG past the
 * last kernel. */
MCGEN_API int mcgen_gb300_profile(int enable);
MCGEN_API int mcgen_gb300_profile_read(int kernel, const char **name, double *total_ms, long long *launches);

/* Last CUDA error text seen by the library (empty when none). */
MCGEN_API const char *mcgen_gb300_last_error(void);

/* Device self-check of the exact integer coordinate split used by every octave sample: n generated
 * inputs (quart coordinates, shifted and second-stack coordinates, tiny/huge values, sums landing on or
 * near integers and in (-1, 0), edge offsets) through both the fast split and the plain double arithmetic
 * of the reference; *bad_f / *bad_d count differing results of the float (26.3) and double (26.1/26.2)
 * branches (the double branch also checks the fraction in units of 2^-52).  Same seed, same inputs. */
MCGEN_API int mcgen_gb300_check_split(long long n, unsigned long long seed, long long *bad_f, long long *bad_d);
/* Device self-check of the double branch's fixed-point octave (gradient sums and first lerp differences in
 * units of 2^-52) against the plain double octave: n random (permutation, fractions) cases; *bad counts
 * results that differ as doubles. */
MCGEN_API int mcgen_gb300_check_octave(long long n, unsigned long long seed, long long *bad);
/* Device self-check of BiomeManager's zoom choice (single-precision screen, double precision only for
 * candidates within its error margin) against the double-precision first minimum of all 8 candidates:
 * n random (zoom seed, block) cases; *bad counts different choices, *screened_out the cases that needed the
 * double-precision comparison. */
MCGEN_API int mcgen_gb300_check_zoom(long long n, unsigned long long seed, long long *bad, long long *screened_out);
/* Device self-check of the double branch's screened climate noises (fixed-point value, exact double only
 * where the float rounding is not settled by the error bound) on the world's own seed lattices: n random
 * coordinates (integer part of magnitude up to 2^25 plus a shift in (-4, 4)), every screened noise of the
 * world (Overworld 26.1/26.2: temperature .. ridge and ridges_folded; Nether: both).  *bad counts floats
 * that differ from the exact path's, *screened_out the values left to the exact path, *worst_ratio the
 * largest |fixed-point - exact| over the bound.  MCGEN_E_ARG for float-branch and End worlds. */
MCGEN_API int mcgen_gb300_check_noise(const McWorld *w, long long n, unsigned long long seed, long long *bad,
                                      long long *screened_out, double *worst_ratio);
/* Device self-check of the double branch's 32-bit screen of the noises whose value is only quantised (the
 * kernels' form for the Nether's two noises; checked on the Overworld's temperature and vegetation as well,
 * whose constants differ), on mcgen_gb300_check_noise's coordinates:
 * *bad counts settled targets that differ from quantize((float)exact), *screened_out the values the screen
 * leaves to the 59-bit screen, *worst_ratio the largest |value - exact| over the bound, *near_boundary the
 * settled values whose exact value lies within twice the bound of a target boundary.  MCGEN_E_ARG for
 * float-branch and End worlds. */
MCGEN_API int mcgen_gb300_check_noise_quant(const McWorld *w, long long n, unsigned long long seed, long long *bad,
                                            long long *screened_out, double *worst_ratio, long long *near_boundary);
/* Device self-check of the double branch's whole Overworld climate as the kernels compute it (exact shift
 * noises, climate noises screened in fixed point) against the plain double evaluation of every noise: n
 * random quart cells (|qx|, |qz| up to 2^21).  *bad counts cells whose six quantised targets differ,
 * *fallback the cells with at least one value the screen left to the exact double path.  MCGEN_E_ARG for
 * float-branch, Nether and End worlds. */
MCGEN_API int mcgen_gb300_check_climate(const McWorld *w, long long n, unsigned long long seed, long long *bad,
                                        long long *fallback);
/* Device self-check of the R-tree searches of a world's tree (Overworld or Nether): the level-unrolled and
 * single-loop searches with 32-bit box distances, and the tie search, against the 64-bit stack searches on
 * n random targets (half of them beyond the 32-bit distances' clamp); and the warp-shared search (one pruned
 * walk per warp of neighbouring cells) on n more targets clustered per warp at several spreads, some lanes
 * inactive, some warps with a lane beyond the packed range.  *bad_leaf counts differing leaves, *bad_other
 * differing fitness values or tie flags.  MCGEN_E_ARG for End worlds. */
MCGEN_API int mcgen_gb300_check_tree(const McWorld *w, long long n, unsigned long long seed, long long *bad_leaf,
                                     long long *bad_other);

/* Device self-check of the End's screened island test (the three simplex corner terms in float, decided when
 * farther from the -0.9 threshold than the float evaluation's error bound, else the exact double value)
 * against the reference's double simplex: n random (permutation, chunk cell) cases, both branches.  *bad
 * counts different decisions, *screened_out the cases left to the exact value, *worst_ratio the largest
 * |float evaluation - double value| over the bound. */
MCGEN_API int mcgen_gb300_check_end(long long n, unsigned long long seed, long long *bad, long long *screened_out,
                                    double *worst_ratio);

/* Pipe microbenchmarks on the current device, in giga-operations per second:
 * 0 FP32 FMA, 1 FP64 FMA, 2 FP64 add, 3 int32 multiply-add, 4 double->int floor conversion,
 * 5 int->double conversion, 6 double->float conversion, 7 64-bit wide integer multiply-add. */
MCGEN_API int mcgen_gb300_pipe_rate(int pipe, double *gops);

#ifdef __cplusplus
}
#endif
#endif
