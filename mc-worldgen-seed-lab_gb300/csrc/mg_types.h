/* mg_types.h -- plain-old-data layouts shared by the host world builder and the sm_103a kernels.
 *
 * Everything here is seed-independent except MgLattice (one Perlin octave of one seed), which the
 * per-seed setup kernel writes and the sampling kernels read.
 */
#ifndef MG_TYPES_H
#define MG_TYPES_H
#include <stdint.h>

#define MG_MAX_OCT 12        /* octaves per NormalNoise stack (continentalness has 9) */
#define MG_OW_NOISES 6       /* offset (shift), temperature, vegetation, continentalness, erosion, ridge */
#define MG_MAX_TABLES 48     /* lattices per seed: Overworld 46, Nether 8, End 1 */
#define MG_SPL_MP 128        /* offset-spline multipoint nodes (26.x: 53) */
#define MG_SPL_PTS 512       /* offset-spline points (26.x: 253) */
#define MG_SPL_CONST 512     /* offset-spline constant leaves (26.x: 201) */
#define MG_SPL_DEPTH 6       /* multipoint levels an offset spline may nest (every 26.x table: 4); the device
                              * evaluator keeps one stack frame per level */
#define MG_TREE_DIMS 7

enum { MG_OVERWORLD = 0, MG_NETHER = 1, MG_END = 2 };
enum { MG_V26_1 = 0, MG_V26_2 = 1, MG_V26_3 = 2, MG_V26_4 = 3 };
/* how equal-fitness leaves resolve (see include/mcgen_gb300.h) */
enum { MG_TIE_ENGINE = 0, MG_TIE_GRID_CHAIN = 1, MG_TIE_CHUNK_CELL = 2, MG_TIE_CHUNK_ORDER = 3 };

/* One NormalNoise, seed-independent.  Level k of stack s uses lattice table base + s*nlev + k. */
typedef struct {
    int32_t nlev;       /* present octaves per stack */
    int32_t legacy;     /* Nether biome noise: LCG init, stack-then-stack summation (float branch) */
    int32_t base;       /* first table index of this noise inside a seed's lattice array */
    int32_t octs;       /* amplitude-array length (legacy init walks it) */
    int32_t first;      /* first octave */
    int32_t idx[MG_MAX_OCT];       /* amplitude index of level k */
    uint64_t hlo[MG_MAX_OCT], hhi[MG_MAX_OCT]; /* md5("octave_<n>") halves */
    double freq[MG_MAX_OCT];       /* input factor of level k, 2^fexp[k] */
    int32_t fexp[MG_MAX_OCT];      /* log2 of freq[k] */
    double amp_d[MG_MAX_OCT];      /* double branch: amplitude */
    double vf_d[MG_MAX_OCT];       /* double branch: value factor of the level */
    double vfac;                   /* double branch: NormalNoise value factor */
    float amp_f[MG_MAX_OCT];       /* float branch: layer amplitude */
    /* double branch, screened evaluation: amp_d[k] * vf_d[k] * vfac times 2^59, and the bound on the
     * difference between the fixed-point value and the reference's double value (< 0: not screened), as a
     * double and in units of 2^-59 (rounded up) */
    int64_t cq[MG_MAX_OCT];
    double fix_err;
    int64_t fix_eq;
    /* double branch, the 32-bit screen of a noise whose value is only quantised (the Nether's two noises):
     * amp_d[k] * vf_d[k] * vfac times 2^31 rounded, and the bound on the difference between its value and the
     * reference's double value in units of 2^-59 (rounded up; < 0: not screened this way) */
    int64_t c31[MG_MAX_OCT];
    int64_t fix_eq32;
} MgNoise;

/* Offset spline (CubicSpline over continents, erosion, ridges, ridges_folded), float.
 * A child reference c >= 0 names multipoint node c; c < 0 names constant ~c. */
typedef struct __attribute__((aligned(16))) {
    int32_t nmp, npt, nconst, root;
    uint8_t coord[MG_SPL_MP];      /* 0 continents, 1 erosion, 2 ridges, 3 ridges_folded */
    uint8_t npts[MG_SPL_MP];
    uint16_t first[MG_SPL_MP];
    float loc[MG_SPL_PTS];
    float der[MG_SPL_PTS];
    int16_t child[MG_SPL_PTS];
    float cval[MG_SPL_CONST];
} MgSpline;

/* R-tree node on the device (32 bytes, two 16-byte loads): children of a subtree are contiguous
 * [first, first+count); a leaf has count == 0.  Bounds of the six climate dimensions are quantised values
 * (|v| <= 12000 in every table), the upper bounds stored negated (nhi = -hi: packed 16-bit add-max
 * instructions then form t - hi); the seventh dimension ("offset") always meets a target coordinate of 0,
 * so its squared distance max(-hi, lo, 0)^2 is stored instead of its bounds.  The root is never a leaf;
 * its biome byte holds MG_TREE_PACKED when every bound lies within +-MG_TREE_PACKED_BOUND (the packed
 * 16-bit distances are then exact for targets within +-(32767 - MG_TREE_PACKED_BOUND)). */
typedef struct __attribute__((aligned(16))) {
    int16_t lo[6];
    int16_t nhi[6];
    uint32_t d7;
    uint16_t first;
    uint8_t count;
    uint8_t biome;
} MgTreeNode;
#define MG_TREE_PACKED 1
#define MG_TREE_PACKED_BOUND 12767

/* Seed-independent world description, copied once to the device. */
typedef struct {
    int32_t version, dim, fmode;   /* fmode 1: float branch (26.3+), 0: double branch */
    int32_t min_y, height;
    int32_t ntables;               /* lattices per seed */
    MgNoise noise[MG_OW_NOISES];   /* Overworld */
    uint64_t nhl[MG_OW_NOISES], nhh[MG_OW_NOISES]; /* md5("minecraft:<noise>") */
    MgNoise nether[2];             /* Nether temperature, vegetation */
    int32_t grad_from_y, grad_to_y;
    double grad_from_d, grad_to_d, off_d;
    double rf_d[3];
    /* ridges_folded's constants times 2^59 and the screen's bound for it in units of 2^-59 (rounded up;
     * < 0: a constant is not a multiple of 2^-59 below 8, and the ridge noise is not screened) */
    int64_t rf_q[3];
    int64_t rf_eq;
    float grad_from_f, grad_to_f, off_f, grad_fac_f;
    float rf_f[3];
    int32_t end_ids[5];            /* the_end, end_highlands, end_midlands, small_end_islands, end_barrens */
    double end_f2, end_g2;         /* 2-D simplex skew 0.5*(sqrt(3)-1) and unskew (3-sqrt(3))/6 */
    int32_t tree_root, tree_nodes, tree_leaves;
    int32_t tree_fanout;           /* most children of a node (the build's children per node: 6 or 19) */
    MgSpline spline;
} MgWorldDesc;

/* Split of the y and z offsets for a zero input coordinate, by branch. */
typedef union {
    struct {
        float fy, fz;  /* (float)fyd, (float)fzd */
        float uy, uz;  /* smoothstep(fy), smoothstep(fz) in float */
    } f;               /* float branch */
    struct {
        int64_t uy, uz; /* smoothstep of Fy, Fz in 2^-59 fixed point (0 where Fy, Fz < 0) */
    } q;                /* double branch (the screened fixed-point evaluation) */
} MgLatZero;

/* One Perlin octave of one seed: offsets, the lattice split of the y and z offsets (what a zero input
 * coordinate uses: fraction and smoothstep of the fraction, and the fraction as a multiple of 2^-52 for
 * the double branch's exact fixed-point gradient sums), and the permutation.
 * 352 bytes, 16-byte aligned; the 96-byte header precedes the permutation. */
typedef struct __attribute__((aligned(16))) {
    double ox, oy, oz;
    double fyd, fzd;   /* oy - floor(oy), oz - floor(oz) (double branch) */
    double uyd, uzd;   /* smoothstep(fyd), smoothstep(fzd) */
    int64_t Fy, Fz;    /* fyd, fzd in units of 2^-52, or -1 when not a multiple of 2^-52 */
    int32_t iy, iz;    /* floor(oy), floor(oz) */
    MgLatZero z0;
    uint8_t p[256];
} MgLattice;

/* A double-branch Overworld cell whose screened climate left a value to the exact double evaluation
 * (about one cell in a thousand): the batch kernel records it here instead of running that evaluation inside
 * a warp whose other lanes would wait for it, and a second kernel finishes the recorded cells densely, one per
 * thread.  72 bytes. */
typedef struct {
    double x, z;      /* the climate noises' input: the cell's shifted coordinates */
    double g;         /* depth gradient at the cell's y */
    int64_t out;      /* output byte of the cell */
    float f[4];       /* temperature, vegetation (a float with the settled target), continentalness, erosion */
    float rv, rf;     /* ridge and ridges_folded floats, when settled */
    int32_t world;    /* index into the batch's world table */
    int32_t state;    /* first lattice of its seed in the state pool */
    uint32_t pend;    /* bit k < 4: climate noise k + 1 unsettled; bit 4: the ridge (with ridges_folded) */
    int32_t pad;
} MgPending;

/* One seed-search observation (the reference's McgObs, engine/cuda/mc_gpu.cuh:47-54): a quart cell, or a
 * block resolved through BiomeManager's zoom when flags has MG_OBS_BLOCK; flags' low byte is the End window
 * half-width; the biomes that satisfy it as a 128-bit mask.  32 bytes. */
typedef struct {
    int32_t qx, qy, qz, flags;
    uint64_t mask[2];
} MgObs;
#define MG_OBS_BLOCK 0x100
#define MG_MAX_OBS 64

#endif
