/* mcgen.h -- drop-in C ABI of libmcgen's biome path, served by hand-written sm_103a kernels.
 *
 * Prototypes, types and error codes are the reference's (libmcgen/include/mcgen.h), so a caller that
 * binds libmcgen (the Blender add-on's ctypes layer, blender/mcgen_addon/core/lib.py:125-126,403-408;
 * libmcgen/tests/g9_biomes.c; mcgen-cli) can load this library instead for biome maps.  Each
 * declaration cites the reference line it replaces.
 *
 * Differences a caller sees:
 *  - mcgen_open's first argument is a data root holding data/climate-<V>.txt and
 *    data/params/<V>/{overworld,nether}.tsv (the reference engine's layout, engine/mc_data.h:84-183),
 *    not a Mojang datapack directory.
 *  - Everything is computed on the GPU; there is no CPU path.  mcgen_biome_grid_cpu and
 *    mcgen_gpu_set_compute(MCGEN_COMPUTE_CPU) return MCGEN_E_UNSUPPORTED, and a missing device makes
 *    biome calls fail loudly (error code, or -1 from mcgen_biome_at) instead of falling back.
 *  - Terrain, regions, structures and tweaks (outside the biome path) return MCGEN_E_UNSUPPORTED or
 *    report zero entries.
 * McGen and McWorld are immutable after creation and safe for concurrent readers; GPU work from
 * concurrent callers is serialised inside the library (libmcgen/gpu/mcgpu_core.cu:12-13).
 */
#ifndef MCGEN_H
#define MCGEN_H
#include <stddef.h>
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif
#if defined(_WIN32)
#define MCGEN_API __declspec(dllexport)
#else
#define MCGEN_API __attribute__((visibility("default")))
#endif

#define MCGEN_ABI_VERSION 1 /* libmcgen/include/mcgen.h:23 */

typedef struct McGen McGen;       /* version data (libmcgen/include/mcgen.h:25) */
typedef struct McWorld McWorld;   /* dimension + preset + seeds (:26) */
typedef struct McRegion McRegion; /* terrain region; never produced here (:27) */

/* libmcgen/include/mcgen.h:29-32 */
enum {
    MCGEN_OK = 0, MCGEN_E_ARG = 1, MCGEN_E_IO = 2, MCGEN_E_DATA = 3, MCGEN_E_VERSION = 4,
    MCGEN_E_NOMEM = 5, MCGEN_E_CANCEL = 6, MCGEN_E_UNSUPPORTED = 7, MCGEN_E_INTERNAL = 8
};
/* libmcgen/include/mcgen.h:44-47 */
enum {
    MC_STAGE_BIOMES = 1u, MC_STAGE_TERRAIN = 2u, MC_STAGE_SURFACE = 4u, MC_STAGE_CARVERS = 8u,
    MC_STAGE_FEATURES = 16u, MC_STAGE_STRUCTURES = 32u, MC_STAGE_ALL = 63u
};

/* libmcgen/include/mcgen.h:50-56.  Only `climate` reaches the biome path. */
typedef struct McSeeds {
    int64_t climate;
    int64_t terrain;
    int64_t structures;
    int64_t features;
} McSeeds;
static inline McSeeds mcgen_seeds_unified(int64_t s) { McSeeds r = {s, s, s, s}; return r; }

/* libmcgen/include/mcgen.h:59-66 */
typedef struct McTweakInfo {
    const char *id, *label, *group, *description;
    double def, min, max, soft_min, soft_max;
    int is_int;
} McTweakInfo;
typedef struct McTweakValue { const char *id; double value; } McTweakValue;
typedef int (*McProgressFn)(void *ud, double fraction, const char *what);

/* ---- version, data (libmcgen/include/mcgen.h:69-87) ---- */
MCGEN_API const char *mcgen_version(void);  /* :69 */
MCGEN_API int mcgen_abi_version(void);      /* :70 */
/* :72.  data_root: directory with data/climate-<V>.txt and data/params/<V>/.  version: "26.1", "26.2",
 * "26.3", "26.4-snapshot-2". */
MCGEN_API int mcgen_open(const char *data_root, const char *version, McGen **out, char *err, size_t errlen);
MCGEN_API void mcgen_close(McGen *g);                                                   /* :73 */
MCGEN_API int mcgen_dimension_count(const McGen *g);                                    /* :75 */
MCGEN_API const char *mcgen_dimension_name(const McGen *g, int i);                      /* :76 */
MCGEN_API int mcgen_preset_count(const McGen *g, const char *dimension);                /* :77 */
MCGEN_API const char *mcgen_preset_name(const McGen *g, const char *dimension, int i);  /* :78 */
MCGEN_API int mcgen_block_state_count(const McGen *g);                                  /* :80, 0 here */
MCGEN_API const char *mcgen_block_state_name(const McGen *g, int id);                   /* :81, NULL */
MCGEN_API int mcgen_block_state_from_name(const McGen *g, const char *name);            /* :82, -1 */
MCGEN_API int mcgen_biome_count(const McGen *g);                                        /* :83 */
MCGEN_API const char *mcgen_biome_name(const McGen *g, int id);                         /* :84 */
MCGEN_API int mcgen_tweak_count(const McGen *g);                                        /* :86, 0 */
MCGEN_API const McTweakInfo *mcgen_tweak_info(const McGen *g, int i);                   /* :87, NULL */

/* ---- world (libmcgen/include/mcgen.h:90-104) ---- */
/* :90-91.  dimension: "minecraft:overworld" | "minecraft:the_nether" | "minecraft:the_end" (or the short
 * forms); preset: "normal" (NULL/""), "amplified", "large_biomes".  Tweaks: none are defined, so any
 * tweak entry is rejected with MCGEN_E_ARG. */
MCGEN_API int mcgen_world_new(McGen *g, const char *dimension, const char *preset, const McSeeds *seeds,
                              const McTweakValue *tweaks, int ntweaks, McWorld **out, char *err, size_t errlen);
MCGEN_API void mcgen_world_free(McWorld *w);                                              /* :92 */
MCGEN_API int mcgen_world_set_schedule(McWorld *w, const char *path, char *err, size_t errlen); /* :96 */
MCGEN_API int mcgen_world_min_y(const McWorld *w);                                        /* :97 */
MCGEN_API int mcgen_world_height(const McWorld *w);                                       /* :98 */
MCGEN_API int mcgen_world_sea_level(const McWorld *w);                                    /* :99 */
/* :102.  Biome id at a block (BiomeManager zoom + chunk-stored tie semantics), -1 on error. */
MCGEN_API int mcgen_biome_at(const McWorld *w, int x, int y, int z);
/* :104.  nx*nz biome ids, out[iz*nx+ix] = biome at (x0+ix*step, y, z0+iz*step). */
MCGEN_API int mcgen_biome_grid(const McWorld *w, int x0, int z0, int nx, int nz, int step, int y, uint8_t *out);

/* ---- terrain region (libmcgen/include/mcgen.h:107-144): outside the biome path ---- */
typedef struct McRegionInfo { int cx0, cz0, nx, nz, min_y, height; } McRegionInfo;
typedef struct McStructureStart {
    const char *id;
    int chunk_x, chunk_z;
    int bb[6];
    int piece_count;
} McStructureStart;
MCGEN_API int mcgen_generate_region(McWorld *w, int cx0, int cz0, int nx, int nz, uint32_t stages, int threads,
                                    McProgressFn cb, void *ud, McRegion **out, char *err, size_t errlen); /* :111 */
MCGEN_API void mcgen_region_free(McRegion *r);                                   /* :113 */
MCGEN_API void mcgen_region_info(const McRegion *r, McRegionInfo *info);         /* :114 */
MCGEN_API uint16_t *mcgen_region_blocks(McRegion *r, int cx, int cz);            /* :116 */
MCGEN_API uint8_t *mcgen_region_biomes(McRegion *r, int cx, int cz);             /* :118 */
MCGEN_API int16_t *mcgen_region_heightmap(McRegion *r, int cx, int cz, int kind); /* :120 */
MCGEN_API int mcgen_region_write_mcr(const McRegion *r, const McGen *g, const char *path, char *err, size_t errlen); /* :123 */
MCGEN_API const char *mcgen_region_block_entities(const McRegion *r);            /* :131 */
MCGEN_API int mcgen_structure_starts(McWorld *w, int cx0, int cz0, int nx, int nz, McStructureStart *out, int cap); /* :142 */
MCGEN_API int mcgen_structure_piece_bb(McWorld *w, int chunk_x, int chunk_z, int index, int piece, int bb[6]); /* :144 */

/* ---- GPU control (libmcgen/include/mcgen.h:149-172) ---- */
enum { MCGEN_COMPUTE_CPU = 0, MCGEN_COMPUTE_GPU = 1, MCGEN_COMPUTE_AUTO = 2 }; /* :149 */
enum { MCGEN_GPU_BIOMES = 1, MCGEN_GPU_TERRAIN = 2 };                           /* :152 */
MCGEN_API int mcgen_gpu_set_features(int mask);                                 /* :153 */
MCGEN_API int mcgen_gpu_get_features(void);                                     /* :154 */
MCGEN_API int mcgen_gpu_set_library_path(const char *path);                     /* :156, kernels are in-library */
MCGEN_API int mcgen_gpu_device_count(void);                                     /* :158 */
MCGEN_API int mcgen_gpu_device_info(int index, char *name, size_t namelen, int *cc_major, int *cc_minor,
                                    size_t *mem_mb);                            /* :159 */
MCGEN_API int mcgen_gpu_set_compute(int mode, int device);                      /* :161 */
MCGEN_API int mcgen_gpu_get_compute(void);                                      /* :162 */
MCGEN_API int mcgen_gpu_status(char *buf, size_t buflen);                       /* :164 */
/* :167.  Compares the device against the device on independent paths (grid vs points) for every
 * dimension and preset of the version; MCGEN_OK when they agree. */
MCGEN_API int mcgen_gpu_selftest(McGen *g, int npoints, char *report, size_t replen);
MCGEN_API int mcgen_gpu_biome_grid(const McWorld *w, int x0, int z0, int nx, int nz, int step, int y, uint8_t *out); /* :169 */
MCGEN_API int mcgen_biome_grid_cpu(const McWorld *w, int x0, int z0, int nx, int nz, int step, int y, uint8_t *out); /* :170 */
/* :172.  Biomes at block points xyz[3n]; *n_cpu is always 0 (no point is handed to a CPU). */
MCGEN_API int mcgen_gpu_biome_points(const McWorld *w, int n, const int *xyz, uint8_t *out, int *n_cpu);

#ifdef __cplusplus
}
#endif
#endif /* MCGEN_H */
