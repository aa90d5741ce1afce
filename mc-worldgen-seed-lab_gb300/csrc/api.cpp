/* api.cpp -- the C ABI (include/mcgen.h, include/mcgen_gb300.h) over the sm_103a kernels.
 *
 * Host side of the drop-in boundary.  McGen holds a version's data root; McWorld holds the seed-independent
 * world description, its device copy (R-tree) and the device lattices of its climate seed, created on the
 * first GPU call.  GPU work from concurrent callers is serialised by one mutex, as the reference's
 * libmcgen_cuda does (libmcgen/gpu/mcgpu_core.cu:12-13).  There is no CPU path: without a device every
 * biome call returns an error (MCGEN_E_UNSUPPORTED) and mcgen_biome_at returns -1.
 */
#include <cuda_runtime.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <atomic>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/mcgen.h"
#include "../../include/mcgen_gb300.h"
#include "abi_internal.h"
#include "launch.h"
#include "prof.h"
#include "world.h"

namespace {

std::mutex g_lock;
int g_mode = MCGEN_COMPUTE_GPU; /* only GPU and Auto (= GPU) are meaningful here */
int g_features = MCGEN_GPU_BIOMES;
int g_device = 0;
int g_dev_state = 0; /* 0 unknown, 1 ready, -1 unavailable */
cudaStream_t g_stream = nullptr;
char g_dev_name[256] = "";
int g_cc_major = 0, g_cc_minor = 0;
size_t g_mem_mb = 0;
thread_local std::string t_last_error;
std::string g_last_cuda;
int g_worlds_ok = 0, g_worlds_failed = 0;
std::string g_selftest = "not run";

void set_err(char *err, size_t errlen, const char *fmt, ...) {
    if (!err || !errlen) return;
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(err, errlen, fmt, ap);
    va_end(ap);
}

int cuda_code(cudaError_t e) {
    if (e == cudaSuccess) return MCGEN_OK;
    g_last_cuda = cudaGetErrorString(e);
    t_last_error = g_last_cuda;
    return e == cudaErrorMemoryAllocation ? MCGEN_E_NOMEM : MCGEN_E_INTERNAL;
}

/* Select and initialise the device once; caller holds g_lock. */
int device_ready_locked() {
    if (g_dev_state == 1) return 1;
    if (g_dev_state == -1) return 0;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n <= 0) {
        cudaGetLastError();
        g_dev_state = -1;
        t_last_error = "no CUDA device";
        return 0;
    }
    if (g_device >= n) g_device = 0;
    cudaDeviceProp p;
    if (cudaSetDevice(g_device) != cudaSuccess || cudaGetDeviceProperties(&p, g_device) != cudaSuccess) {
        g_dev_state = -1;
        t_last_error = "cannot use CUDA device";
        return 0;
    }
    snprintf(g_dev_name, sizeof g_dev_name, "%s", p.name);
    g_cc_major = p.major;
    g_cc_minor = p.minor;
    g_mem_mb = p.totalGlobalMem >> 20;
    if (cudaStreamCreateWithFlags(&g_stream, cudaStreamNonBlocking) != cudaSuccess) {
        g_dev_state = -1;
        t_last_error = "cannot create a CUDA stream";
        return 0;
    }
    /* keep freed stream-ordered scratch cached in the pool instead of returning it to the driver */
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, g_device) == cudaSuccess) {
        uint64_t keep = ~0ULL;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
    g_dev_state = 1;
    return 1;
}

/* Device copies of a world (tree + its seed's lattices); caller holds g_lock and a ready device. */
int world_device_locked(McWorld *w) {
    if (w->dev_ready) return MCGEN_OK;
    cudaError_t e = cudaSuccess;
    size_t tb = sizeof(MgTreeNode) * (w->tree.empty() ? 1 : w->tree.size());
    if ((e = cudaMalloc(&w->d_tree, tb)) != cudaSuccess) return cuda_code(e);
    if (!w->tree.empty() && (e = cudaMemcpy(w->d_tree, w->tree.data(), sizeof(MgTreeNode) * w->tree.size(),
                                            cudaMemcpyHostToDevice)) != cudaSuccess)
        return cuda_code(e);
    if ((e = cudaMalloc(&w->d_state, sizeof(MgLattice) * (size_t)w->desc.ntables)) != cudaSuccess) return cuda_code(e);
    int64_t *d_seed = nullptr;
    if ((e = cudaMallocAsync(&d_seed, sizeof(int64_t), g_stream)) != cudaSuccess) return cuda_code(e);
    cudaMemcpyAsync(d_seed, &w->seeds.climate, sizeof(int64_t), cudaMemcpyHostToDevice, g_stream);
    int rc = mg::launch_setup(w->desc, d_seed, 1, w->d_state, g_stream);
    cudaFreeAsync(d_seed, g_stream);
    if (rc) return cuda_code((cudaError_t)rc);
    if ((e = cudaStreamSynchronize(g_stream)) != cudaSuccess) return cuda_code(e);
    w->dev_ready = 1;
    return MCGEN_OK;
}

/* cudaFree waits for the device work that may still read the tree */
void world_destroy_locked(McWorld *w) {
    if (w->d_tree) cudaFree(w->d_tree);
    if (w->d_state) cudaFree(w->d_state);
    delete w;
}

std::atomic<uint64_t> g_world_uid{1};

int dim_of(const char *d) {
    if (!d) return -1;
    if (!strcmp(d, "minecraft:overworld") || !strcmp(d, "overworld")) return MG_OVERWORLD;
    if (!strcmp(d, "minecraft:the_nether") || !strcmp(d, "the_nether") || !strcmp(d, "nether")) return MG_NETHER;
    if (!strcmp(d, "minecraft:the_end") || !strcmp(d, "the_end") || !strcmp(d, "end")) return MG_END;
    return -1;
}
const char *dim_name(int d) {
    static const char *const n[3] = {"minecraft:overworld", "minecraft:the_nether", "minecraft:the_end"};
    return (d >= 0 && d < 3) ? n[d] : nullptr;
}

struct DevBuf { /* stream-ordered scratch, freed on the same stream */
    void *p = nullptr;
    cudaStream_t s;
    explicit DevBuf(cudaStream_t st) : s(st) {}
    cudaError_t alloc(size_t n) { return n ? cudaMallocAsync(&p, n, s) : cudaSuccess; }
    ~DevBuf() { if (p) cudaFreeAsync(p, s); }
};

/* End chunk-class table bounds for block samples x in [xmin, xmax], z in [zmin, zmax]: the zoom picks the
 * quart cell (x-2)>>2 or one more, and a quart cell q lies in chunk q>>2. */
void end_chunk_range(long long xmin, long long xmax, long long zmin, long long zmax, int *cx0, int *cz0, int *ncx,
                     int *ncz) {
    long long qx0 = (xmin - 2) >> 2, qx1 = ((xmax - 2) >> 2) + 1, qz0 = (zmin - 2) >> 2, qz1 = ((zmax - 2) >> 2) + 1;
    *cx0 = (int)(qx0 >> 2);
    *cz0 = (int)(qz0 >> 2);
    *ncx = (int)((qx1 >> 2) - (qx0 >> 2) + 1);
    *ncz = (int)((qz1 >> 2) - (qz0 >> 2) + 1);
}

/* Block-coordinate biomes into device memory on `st` (grid or point list). */
int block_biomes_dev(const McWorld *w, int x0, int z0, int nx, int nz, int step, int y, const int32_t *d_xyz,
                     long long xmin, long long xmax, long long zmin, long long zmax, uint8_t *d_out, cudaStream_t st) {
    int cx0 = 0, cz0 = 0, ncx = 0, ncz = 0;
    DevBuf cls(st);
    const long long n = (long long)nx * nz;
    if (w->desc.dim == MG_END) {
        end_chunk_range(xmin, xmax, zmin, zmax, &cx0, &cz0, &ncx, &ncz);
        /* a table is worth it when samples share chunks; sparse samples evaluate their chunk directly */
        if ((long long)ncx * ncz <= 4 * n + 4096) {
            cudaError_t e = cls.alloc((size_t)ncx * (size_t)ncz);
            if (e) return cuda_code(e);
        }
    }
    int rc = mg::launch_block_biomes(w->desc, w->d_tree, w->d_state, w->zoom_seed, x0, z0, nx, nz, step, y, d_xyz,
                                     d_out, cls.p, cx0, cz0, ncx, ncz, st);
    return rc ? cuda_code((cudaError_t)rc) : MCGEN_OK;
}

}  // namespace

namespace mg {
std::mutex &abi_lock() { return g_lock; }
int abi_device() { return g_device; }
int abi_device_ready() { return device_ready_locked(); }
cudaStream_t abi_stream() { return g_stream; }
int abi_world_device(McWorld *w) { return world_device_locked(w); }
int abi_cuda_code(int e) { return cuda_code((cudaError_t)e); }
void abi_world_hold(McWorld *w) { w->holds++; }
void abi_world_release(McWorld *w) {
    if (w->holds > 0) w->holds--;
    if (w->holds == 0 && w->free_requested) world_destroy_locked(w);
}
}  // namespace mg

/* ============================================================================ version, data */
extern "C" {

MCGEN_API const char *mcgen_version(void) { return "libmcgen-gb300 0.1.0 abi 1"; }
MCGEN_API int mcgen_abi_version(void) { return MCGEN_ABI_VERSION; }

MCGEN_API int mcgen_open(const char *data_root, const char *version, McGen **out, char *err, size_t errlen) {
    if (!data_root || !version || !out) { set_err(err, errlen, "mcgen_open: null argument"); return MCGEN_E_ARG; }
    *out = nullptr;
    int v = mg::version_from_name(version);
    if (v < 0) { set_err(err, errlen, "unknown version %s", version); return MCGEN_E_VERSION; }
    std::string path = std::string(data_root) + "/data/climate-" + mg::version_name(v) + ".txt";
    FILE *f = fopen(path.c_str(), "rb");
    if (!f) { set_err(err, errlen, "cannot read %s", path.c_str()); return MCGEN_E_IO; }
    fclose(f);
    McGen *g = new (std::nothrow) McGen;
    if (!g) return MCGEN_E_NOMEM;
    g->version = v;
    g->root = data_root;
    *out = g;
    return MCGEN_OK;
}
MCGEN_API void mcgen_close(McGen *g) { delete g; }

MCGEN_API int mcgen_dimension_count(const McGen *g) { return g ? 3 : 0; }
MCGEN_API const char *mcgen_dimension_name(const McGen *g, int i) { return g ? dim_name(i) : nullptr; }
MCGEN_API int mcgen_preset_count(const McGen *g, const char *dimension) {
    return g ? mg::preset_count(dim_of(dimension)) : 0;
}
MCGEN_API const char *mcgen_preset_name(const McGen *g, const char *dimension, int i) {
    return g ? mg::preset_name(dim_of(dimension), i) : nullptr;
}
MCGEN_API int mcgen_block_state_count(const McGen *g) { (void)g; return 0; }
MCGEN_API const char *mcgen_block_state_name(const McGen *g, int id) { (void)g; (void)id; return nullptr; }
MCGEN_API int mcgen_block_state_from_name(const McGen *g, const char *name) { (void)g; (void)name; return -1; }
MCGEN_API int mcgen_biome_count(const McGen *g) { return g ? mg::biome_count() : 0; }
MCGEN_API const char *mcgen_biome_name(const McGen *g, int id) {
    static std::vector<std::string> names;
    static std::once_flag once;
    std::call_once(once, [] {
        for (int i = 0; i < mg::biome_count(); i++) names.push_back(std::string("minecraft:") + mg::biome_key(i));
    });
    return (g && id >= 0 && id < (int)names.size()) ? names[(size_t)id].c_str() : nullptr;
}
MCGEN_API int mcgen_tweak_count(const McGen *g) { (void)g; return 0; }
MCGEN_API const McTweakInfo *mcgen_tweak_info(const McGen *g, int i) { (void)g; (void)i; return nullptr; }

/* ============================================================================ world */
MCGEN_API int mcgen_world_new(McGen *g, const char *dimension, const char *preset, const McSeeds *seeds,
                              const McTweakValue *tweaks, int ntweaks, McWorld **out, char *err, size_t errlen) {
    if (!g || !dimension || !seeds || !out) { set_err(err, errlen, "mcgen_world_new: null argument"); return MCGEN_E_ARG; }
    *out = nullptr;
    int d = dim_of(dimension);
    if (d < 0) { set_err(err, errlen, "unknown dimension %s", dimension); return MCGEN_E_ARG; }
    std::string pn = (preset && *preset) ? preset : "normal";
    if (pn.compare(0, 10, "minecraft:") == 0) pn = pn.substr(10);
    bool known = false;
    for (int i = 0; i < mg::preset_count(d); i++) known |= pn == mg::preset_name(d, i);
    if (!known) { set_err(err, errlen, "no preset %s for %s", pn.c_str(), dimension); return MCGEN_E_ARG; }
    if (ntweaks > 0 && tweaks) {
        set_err(err, errlen, "unknown tweak %s", tweaks[0].id ? tweaks[0].id : "(null)");
        return MCGEN_E_ARG;
    }
    McWorld *w = new (std::nothrow) McWorld();
    if (!w) return MCGEN_E_NOMEM;
    w->g = g;
    w->dim = d;
    w->preset = pn;
    w->seeds = *seeds;
    w->zoom_seed = mg::obfuscate_seed(seeds->climate);
    w->uid = g_world_uid.fetch_add(1);
    std::string e;
    int rc = mg::build_world(g->root.c_str(), g->version, d, pn.c_str(), &w->desc, &w->tree, &e);
    if (rc) {
        set_err(err, errlen, "%s", e.c_str());
        delete w;
        return rc;
    }
    *out = w;
    return MCGEN_OK;
}
/* A world that a plan or a pending served request still uses is freed when the last of them lets go
 * (mg::abi_world_release); its handle is invalid for the caller from this call on either way. */
MCGEN_API void mcgen_world_free(McWorld *w) {
    if (!w) return;
    std::lock_guard<std::mutex> lk(g_lock);
    if (w->holds > 0) {
        w->free_requested = 1;
        return;
    }
    world_destroy_locked(w);
}
MCGEN_API int mcgen_world_set_schedule(McWorld *w, const char *path, char *err, size_t errlen) {
    (void)w; (void)path;
    set_err(err, errlen, "decoration schedules belong to terrain generation, which this library does not provide");
    return MCGEN_E_UNSUPPORTED;
}
MCGEN_API int mcgen_world_min_y(const McWorld *w) { return w ? w->desc.min_y : 0; }
MCGEN_API int mcgen_world_height(const McWorld *w) { return w ? w->desc.height : 0; }
MCGEN_API int mcgen_world_sea_level(const McWorld *w) {
    return w ? (w->dim == MG_OVERWORLD ? 63 : w->dim == MG_NETHER ? 32 : 0) : 0;
}

/* ============================================================================ biomes */
static int grid_common(const McWorld *w, int x0, int z0, int nx, int nz, int step, int y, uint8_t *out) {
    if (!w || !out || nx <= 0 || nz <= 0 || step <= 0) return MCGEN_E_ARG;
    if ((long long)nx * nz > (1LL << 31)) return MCGEN_E_ARG;
    std::lock_guard<std::mutex> lk(g_lock);
    if (!device_ready_locked()) return MCGEN_E_UNSUPPORTED;
    int rc = world_device_locked(const_cast<McWorld *>(w));
    if (rc) return rc;
    const size_t n = (size_t)nx * (size_t)nz;
    DevBuf d_out(g_stream);
    cudaError_t e = d_out.alloc(n);
    if (e) return cuda_code(e);
    long long x1 = (long long)x0 + (long long)(nx - 1) * step, z1 = (long long)z0 + (long long)(nz - 1) * step;
    if (x1 > INT32_MAX || z1 > INT32_MAX) return MCGEN_E_ARG;
    rc = block_biomes_dev(w, x0, z0, nx, nz, step, y, nullptr, x0, x1, z0, z1, (uint8_t *)d_out.p, g_stream);
    if (rc) return rc;
    if ((e = cudaMemcpyAsync(out, d_out.p, n, cudaMemcpyDeviceToHost, g_stream)) != cudaSuccess) return cuda_code(e);
    return cuda_code(cudaStreamSynchronize(g_stream));
}

MCGEN_API int mcgen_biome_grid(const McWorld *w, int x0, int z0, int nx, int nz, int step, int y, uint8_t *out) {
    return grid_common(w, x0, z0, nx, nz, step, y, out);
}
MCGEN_API int mcgen_gpu_biome_grid(const McWorld *w, int x0, int z0, int nx, int nz, int step, int y, uint8_t *out) {
    return grid_common(w, x0, z0, nx, nz, step, y, out);
}
MCGEN_API int mcgen_biome_grid_cpu(const McWorld *w, int x0, int z0, int nx, int nz, int step, int y, uint8_t *out) {
    (void)w; (void)x0; (void)z0; (void)nx; (void)nz; (void)step; (void)y; (void)out;
    t_last_error = "this library computes biomes on the GPU only";
    return MCGEN_E_UNSUPPORTED;
}

MCGEN_API int mcgen_gpu_biome_points(const McWorld *w, int n, const int *xyz, uint8_t *out, int *n_cpu) {
    if (n_cpu) *n_cpu = 0;
    if (!w || n < 0 || (n > 0 && (!xyz || !out))) return MCGEN_E_ARG;
    if (n == 0) return MCGEN_OK;
    long long xmin = xyz[0], xmax = xyz[0], zmin = xyz[2], zmax = xyz[2];
    for (int i = 1; i < n; i++) {
        xmin = xmin < xyz[3 * i] ? xmin : xyz[3 * i];
        xmax = xmax > xyz[3 * i] ? xmax : xyz[3 * i];
        zmin = zmin < xyz[3 * i + 2] ? zmin : xyz[3 * i + 2];
        zmax = zmax > xyz[3 * i + 2] ? zmax : xyz[3 * i + 2];
    }
    std::lock_guard<std::mutex> lk(g_lock);
    if (!device_ready_locked()) return MCGEN_E_UNSUPPORTED;
    int rc = world_device_locked(const_cast<McWorld *>(w));
    if (rc) return rc;
    DevBuf d_xyz(g_stream), d_out(g_stream);
    cudaError_t e;
    if ((e = d_xyz.alloc(sizeof(int32_t) * 3 * (size_t)n)) || (e = d_out.alloc((size_t)n))) return cuda_code(e);
    if ((e = cudaMemcpyAsync(d_xyz.p, xyz, sizeof(int32_t) * 3 * (size_t)n, cudaMemcpyHostToDevice, g_stream))) return cuda_code(e);
    rc = block_biomes_dev(w, 0, 0, n, 1, 1, 0, (const int32_t *)d_xyz.p, xmin, xmax, zmin, zmax, (uint8_t *)d_out.p, g_stream);
    if (rc) return rc;
    if ((e = cudaMemcpyAsync(out, d_out.p, (size_t)n, cudaMemcpyDeviceToHost, g_stream))) return cuda_code(e);
    return cuda_code(cudaStreamSynchronize(g_stream));
}

MCGEN_API int mcgen_biome_at(const McWorld *w, int x, int y, int z) {
    int xyz[3] = {x, y, z};
    uint8_t b = 0;
    return mcgen_gpu_biome_points(w, 1, xyz, &b, nullptr) == MCGEN_OK ? (int)b : -1;
}

/* ============================================================================ terrain (outside the biome path) */
MCGEN_API int mcgen_generate_region(McWorld *w, int cx0, int cz0, int nx, int nz, uint32_t stages, int threads,
                                    McProgressFn cb, void *ud, McRegion **out, char *err, size_t errlen) {
    (void)w; (void)cx0; (void)cz0; (void)nx; (void)nz; (void)stages; (void)threads; (void)cb; (void)ud;
    if (out) *out = nullptr;
    set_err(err, errlen, "terrain regions are not provided by this library (biome path only)");
    return MCGEN_E_UNSUPPORTED;
}
MCGEN_API void mcgen_region_free(McRegion *r) { (void)r; }
MCGEN_API void mcgen_region_info(const McRegion *r, McRegionInfo *info) {
    (void)r;
    if (info) memset(info, 0, sizeof *info);
}
MCGEN_API uint16_t *mcgen_region_blocks(McRegion *r, int cx, int cz) { (void)r; (void)cx; (void)cz; return nullptr; }
MCGEN_API uint8_t *mcgen_region_biomes(McRegion *r, int cx, int cz) { (void)r; (void)cx; (void)cz; return nullptr; }
MCGEN_API int16_t *mcgen_region_heightmap(McRegion *r, int cx, int cz, int kind) {
    (void)r; (void)cx; (void)cz; (void)kind;
    return nullptr;
}
MCGEN_API int mcgen_region_write_mcr(const McRegion *r, const McGen *g, const char *path, char *err, size_t errlen) {
    (void)r; (void)g; (void)path;
    set_err(err, errlen, "terrain regions are not provided by this library");
    return MCGEN_E_UNSUPPORTED;
}
MCGEN_API const char *mcgen_region_block_entities(const McRegion *r) { (void)r; return nullptr; }
MCGEN_API int mcgen_structure_starts(McWorld *w, int cx0, int cz0, int nx, int nz, McStructureStart *out, int cap) {
    (void)w; (void)cx0; (void)cz0; (void)nx; (void)nz; (void)out; (void)cap;
    return 0;
}
MCGEN_API int mcgen_structure_piece_bb(McWorld *w, int chunk_x, int chunk_z, int index, int piece, int bb[6]) {
    (void)w; (void)chunk_x; (void)chunk_z; (void)index; (void)piece; (void)bb;
    return MCGEN_E_UNSUPPORTED;
}

/* ============================================================================ GPU control */
MCGEN_API int mcgen_gpu_set_features(int mask) {
    std::lock_guard<std::mutex> lk(g_lock);
    g_features = mask & (MCGEN_GPU_BIOMES | MCGEN_GPU_TERRAIN);
    return MCGEN_OK;
}
MCGEN_API int mcgen_gpu_get_features(void) { return g_features; }
MCGEN_API int mcgen_gpu_set_library_path(const char *path) { (void)path; return MCGEN_OK; }
MCGEN_API int mcgen_gpu_device_count(void) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) { cudaGetLastError(); return 0; }
    return n;
}
MCGEN_API int mcgen_gpu_device_info(int index, char *name, size_t namelen, int *cc_major, int *cc_minor,
                                    size_t *mem_mb) {
    cudaDeviceProp p;
    if (cudaGetDeviceProperties(&p, index) != cudaSuccess) { cudaGetLastError(); return MCGEN_E_ARG; }
    if (name && namelen) snprintf(name, namelen, "%s", p.name);
    if (cc_major) *cc_major = p.major;
    if (cc_minor) *cc_minor = p.minor;
    if (mem_mb) *mem_mb = p.totalGlobalMem >> 20;
    return MCGEN_OK;
}
MCGEN_API int mcgen_gpu_set_compute(int mode, int device) {
    if (mode == MCGEN_COMPUTE_CPU) {
        t_last_error = "this library computes biomes on the GPU only";
        return MCGEN_E_UNSUPPORTED;
    }
    if (mode != MCGEN_COMPUTE_GPU && mode != MCGEN_COMPUTE_AUTO) return MCGEN_E_ARG;
    std::lock_guard<std::mutex> lk(g_lock);
    if (device >= 0) {
        if (g_dev_state == 1 && device != g_device) return MCGEN_E_UNSUPPORTED; /* device fixed after first use */
        g_device = device;
    }
    g_mode = mode;
    return MCGEN_OK;
}
MCGEN_API int mcgen_gpu_get_compute(void) { return g_mode; }
MCGEN_API int mcgen_gpu_status(char *buf, size_t buflen) {
    std::lock_guard<std::mutex> lk(g_lock);
    int ok = device_ready_locked();
    char line[1024];
    if (ok)
        snprintf(line, sizeof line,
                 "mode: %s\nstate: GPU ready\nfeatures: biomes\ndevice: %s (sm_%d%d, %zu MB)\nlibrary: in-process\n"
                 "worlds_ok: %d\nworlds_failed: %d\nlast_fallback: -\nselftest: %s",
                 g_mode == MCGEN_COMPUTE_AUTO ? "Auto" : "GPU", g_dev_name, g_cc_major, g_cc_minor, g_mem_mb, g_worlds_ok,
                 g_worlds_failed, g_selftest.c_str());
    else
        snprintf(line, sizeof line, "mode: %s\nstate: GPU unavailable (no CPU path in this library)\nreason: %s",
                 g_mode == MCGEN_COMPUTE_AUTO ? "Auto" : "GPU", t_last_error.empty() ? "unknown" : t_last_error.c_str());
    if (buf && buflen) snprintf(buf, buflen, "%s", line);
    return ok;
}

MCGEN_API int mcgen_gpu_selftest(McGen *g, int npoints, char *report, size_t replen);

/* ============================================================================ additions (mcgen_gb300.h) */
MCGEN_API int mcgen_gb300_world_info(const McWorld *w, int *version, int *dimension, int64_t *climate_seed,
                                     int *float_branch) {
    if (!w) return MCGEN_E_ARG;
    if (version) *version = w->desc.version;
    if (dimension) *dimension = w->dim;
    if (climate_seed) *climate_seed = w->seeds.climate;
    if (float_branch) *float_branch = w->desc.fmode;
    return MCGEN_OK;
}

static int quart_grid_on(const McWorld *w, int qx0, int qz0, int nx, int nz, int qy, int rule, uint8_t *d_out,
                         cudaStream_t st) {
    const long long n = (long long)nx * nz;
    DevBuf scratch(st);
    size_t sb = 0;
    if (w->dim == MG_END) sb = (size_t)(nx / 4 + 3) * (size_t)(nz / 4 + 3);
    else if (rule == MCGEN_TIE_GRID_CHAIN || rule == MCGEN_TIE_CHUNK_ORDER) sb = mg::chain_scratch_bytes(n);
    cudaError_t e = scratch.alloc(sb);
    if (e) return cuda_code(e);
    int rc = mg::launch_quart_grid(w->desc, w->d_tree, w->d_state, qx0, qz0, nx, nz, qy, rule, d_out, scratch.p, st);
    return rc ? cuda_code((cudaError_t)rc) : MCGEN_OK;
}

MCGEN_API int mcgen_gb300_quart_grid(const McWorld *w, int qx0, int qz0, int nx, int nz, int qy, int tie_rule,
                                     uint8_t *out) {
    if (!w || !out || nx <= 0 || nz <= 0) return MCGEN_E_ARG;
    if (tie_rule != MCGEN_TIE_ENGINE && tie_rule != MCGEN_TIE_GRID_CHAIN && tie_rule != MCGEN_TIE_CHUNK_ORDER) return MCGEN_E_ARG;
    if ((long long)nx * nz > (1LL << 31)) return MCGEN_E_ARG;
    std::lock_guard<std::mutex> lk(g_lock);
    if (!device_ready_locked()) return MCGEN_E_UNSUPPORTED;
    int rc = world_device_locked(const_cast<McWorld *>(w));
    if (rc) return rc;
    DevBuf d_out(g_stream);
    cudaError_t e = d_out.alloc((size_t)nx * (size_t)nz);
    if (e) return cuda_code(e);
    rc = quart_grid_on(w, qx0, qz0, nx, nz, qy, tie_rule, (uint8_t *)d_out.p, g_stream);
    if (rc) return rc;
    if ((e = cudaMemcpyAsync(out, d_out.p, (size_t)nx * (size_t)nz, cudaMemcpyDeviceToHost, g_stream))) return cuda_code(e);
    return cuda_code(cudaStreamSynchronize(g_stream));
}

MCGEN_API int mcgen_gb300_quart_grid_dev(const McWorld *w, int qx0, int qz0, int nx, int nz, int qy, int tie_rule,
                                         uint8_t *d_out, void *stream) {
    if (!w || !d_out || nx <= 0 || nz <= 0) return MCGEN_E_ARG;
    if (tie_rule != MCGEN_TIE_ENGINE && tie_rule != MCGEN_TIE_GRID_CHAIN && tie_rule != MCGEN_TIE_CHUNK_ORDER) return MCGEN_E_ARG;
    std::lock_guard<std::mutex> lk(g_lock);
    if (!device_ready_locked()) return MCGEN_E_UNSUPPORTED;
    int rc = world_device_locked(const_cast<McWorld *>(w));
    if (rc) return rc;
    return quart_grid_on(w, qx0, qz0, nx, nz, qy, tie_rule, d_out, (cudaStream_t)stream);
}

static int seed_points_on(const McWorld *w, const int64_t *d_seeds, int ns, const int32_t *d_pts, int np,
                          uint8_t *d_out, int32_t *d_tg, cudaStream_t st) {
    if (mg::fused_supported(w->desc)) { /* Overworld: lattices built and sampled on chip */
        DevBuf clim(st);
        cudaError_t e = clim.alloc(mg::fused_scratch_bytes(w->desc, (long long)ns * np));
        if (e) return cuda_code(e);
        int rc = mg::launch_ow_seed_points(w->desc, w->d_tree, d_seeds, ns, d_pts, np, d_out, d_tg, clim.p, st);
        return rc ? cuda_code((cudaError_t)rc) : MCGEN_OK;
    }
    DevBuf states(st);
    cudaError_t e = states.alloc(sizeof(MgLattice) * (size_t)ns * (size_t)w->desc.ntables);
    if (e) return cuda_code(e);
    int rc = mg::launch_setup(w->desc, d_seeds, ns, (MgLattice *)states.p, st);
    if (!rc) rc = mg::launch_points(w->desc, w->d_tree, (const MgLattice *)states.p, ns, d_pts, np, d_out, d_tg, st);
    return rc ? cuda_code((cudaError_t)rc) : MCGEN_OK;
}

MCGEN_API int mcgen_gb300_seed_points(const McWorld *w, const int64_t *seeds, int ns, const int32_t *qxyz, int np,
                                      uint8_t *out, int32_t *targets) {
    if (!w || ns < 0 || np < 0 || (ns > 0 && !seeds) || (np > 0 && (!qxyz || !out))) return MCGEN_E_ARG;
    if ((long long)ns * np == 0) return MCGEN_OK;
    if ((long long)ns * np > (1LL << 31)) return MCGEN_E_ARG;
    std::lock_guard<std::mutex> lk(g_lock);
    if (!device_ready_locked()) return MCGEN_E_UNSUPPORTED;
    int rc = world_device_locked(const_cast<McWorld *>(w));
    if (rc) return rc;
    const size_t n = (size_t)ns * (size_t)np;
    DevBuf d_seeds(g_stream), d_pts(g_stream), d_out(g_stream), d_tg(g_stream);
    cudaError_t e;
    if ((e = d_seeds.alloc(sizeof(int64_t) * (size_t)ns)) || (e = d_pts.alloc(sizeof(int32_t) * 3 * (size_t)np)) ||
        (e = d_out.alloc(n)) || (e = d_tg.alloc(targets ? sizeof(int32_t) * 6 * n : 0)))
        return cuda_code(e);
    if ((e = cudaMemcpyAsync(d_seeds.p, seeds, sizeof(int64_t) * (size_t)ns, cudaMemcpyHostToDevice, g_stream)) ||
        (e = cudaMemcpyAsync(d_pts.p, qxyz, sizeof(int32_t) * 3 * (size_t)np, cudaMemcpyHostToDevice, g_stream)))
        return cuda_code(e);
    rc = seed_points_on(w, (const int64_t *)d_seeds.p, ns, (const int32_t *)d_pts.p, np, (uint8_t *)d_out.p,
                        (int32_t *)d_tg.p, g_stream);
    if (rc) return rc;
    if ((e = cudaMemcpyAsync(out, d_out.p, n, cudaMemcpyDeviceToHost, g_stream))) return cuda_code(e);
    if (targets && (e = cudaMemcpyAsync(targets, d_tg.p, sizeof(int32_t) * 6 * n, cudaMemcpyDeviceToHost, g_stream)))
        return cuda_code(e);
    return cuda_code(cudaStreamSynchronize(g_stream));
}

/* Overworld density functions at block points for an explicit seed (host buffers, synchronous). */
MCGEN_API int mcgen_gb300_density_values(const McWorld *w, int64_t seed, int n, const int32_t *xyz, double *out) {
    if (!w || n < 0 || (n > 0 && (!xyz || !out)) || n > (1 << 28)) return MCGEN_E_ARG;
    if (w->desc.dim != MG_OVERWORLD) return MCGEN_E_ARG;
    if (n == 0) return MCGEN_OK;
    std::lock_guard<std::mutex> lk(g_lock);
    if (!device_ready_locked()) return MCGEN_E_UNSUPPORTED;
    int rc = world_device_locked(const_cast<McWorld *>(w));
    if (rc) return rc;
    cudaError_t e;
    {
        DevBuf d_seed(g_stream), d_lat(g_stream), d_xyz(g_stream), d_out(g_stream);
        if ((e = d_seed.alloc(sizeof(int64_t))) || (e = d_lat.alloc(sizeof(MgLattice) * (size_t)w->desc.ntables)) ||
            (e = d_xyz.alloc(sizeof(int32_t) * 3 * (size_t)n)) || (e = d_out.alloc(sizeof(double) * 5 * (size_t)n)))
            return cuda_code(e);
        if ((e = cudaMemcpyAsync(d_seed.p, &seed, sizeof(int64_t), cudaMemcpyHostToDevice, g_stream)) ||
            (e = cudaMemcpyAsync(d_xyz.p, xyz, sizeof(int32_t) * 3 * (size_t)n, cudaMemcpyHostToDevice, g_stream)))
            return cuda_code(e);
        rc = mg::launch_setup(w->desc, (const int64_t *)d_seed.p, 1, (MgLattice *)d_lat.p, g_stream);
        if (!rc) rc = mg::launch_density(w->desc, (const MgLattice *)d_lat.p, n, (const int32_t *)d_xyz.p,
                                         (double *)d_out.p, g_stream);
        if (rc) return cuda_code((cudaError_t)rc);
        if ((e = cudaMemcpyAsync(out, d_out.p, sizeof(double) * 5 * (size_t)n, cudaMemcpyDeviceToHost, g_stream)))
            return cuda_code(e);
    }
    return cuda_code(cudaStreamSynchronize(g_stream));
}

MCGEN_API int mcgen_gb300_seed_points_dev(const McWorld *w, const int64_t *d_seeds, int ns, const int32_t *d_qxyz,
                                          int np, uint8_t *d_out, int32_t *d_targets, void *stream) {
    if (!w || ns < 0 || np < 0 || (ns > 0 && !d_seeds) || (np > 0 && (!d_qxyz || !d_out))) return MCGEN_E_ARG;
    if ((long long)ns * np == 0) return MCGEN_OK;
    if ((long long)ns * np > (1LL << 31)) return MCGEN_E_ARG;
    std::lock_guard<std::mutex> lk(g_lock);
    if (!device_ready_locked()) return MCGEN_E_UNSUPPORTED;
    int rc = world_device_locked(const_cast<McWorld *>(w));
    if (rc) return rc;
    return seed_points_on(w, d_seeds, ns, d_qxyz, np, d_out, d_targets, (cudaStream_t)stream);
}

MCGEN_API int mcgen_gb300_biome_grid_dev(const McWorld *w, int x0, int z0, int nx, int nz, int step, int y,
                                         uint8_t *d_out, void *stream) {
    if (!w || !d_out || nx <= 0 || nz <= 0 || step <= 0) return MCGEN_E_ARG;
    long long x1 = (long long)x0 + (long long)(nx - 1) * step, z1 = (long long)z0 + (long long)(nz - 1) * step;
    if (x1 > INT32_MAX || z1 > INT32_MAX || (long long)nx * nz > (1LL << 31)) return MCGEN_E_ARG;
    std::lock_guard<std::mutex> lk(g_lock);
    if (!device_ready_locked()) return MCGEN_E_UNSUPPORTED;
    int rc = world_device_locked(const_cast<McWorld *>(w));
    if (rc) return rc;
    return block_biomes_dev(w, x0, z0, nx, nz, step, y, nullptr, x0, x1, z0, z1, d_out, (cudaStream_t)stream);
}

/* One request the plain way: its seed's lattices into stream-ordered scratch, then one grid launch. */
MCGEN_API int mcgen_gb300_quart_grid_seed_dev(const McWorld *w, int64_t seed, int qx0, int qz0, int nx, int nz, int qy,
                                              int tie_rule, uint8_t *d_out, void *stream) {
    if (!w || !d_out || nx <= 0 || nz <= 0) return MCGEN_E_ARG;
    if (tie_rule != MCGEN_TIE_ENGINE && tie_rule != MCGEN_TIE_GRID_CHAIN && tie_rule != MCGEN_TIE_CHUNK_ORDER) return MCGEN_E_ARG;
    std::lock_guard<std::mutex> lk(g_lock);
    if (!device_ready_locked()) return MCGEN_E_UNSUPPORTED;
    int rc = world_device_locked(const_cast<McWorld *>(w));
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    DevBuf state(st), d_seed(st), scratch(st);
    cudaError_t e;
    if ((e = state.alloc(sizeof(MgLattice) * (size_t)w->desc.ntables)) || (e = d_seed.alloc(sizeof(int64_t))))
        return cuda_code(e);
    if ((e = cudaMemcpyAsync(d_seed.p, &seed, sizeof seed, cudaMemcpyHostToDevice, st))) return cuda_code(e);
    if ((rc = mg::launch_setup(w->desc, (const int64_t *)d_seed.p, 1, (MgLattice *)state.p, st))) return cuda_code((cudaError_t)rc);
    size_t sb = 0;
    if (w->dim == MG_END) sb = (size_t)(nx / 4 + 3) * (size_t)(nz / 4 + 3);
    else if (tie_rule == MCGEN_TIE_GRID_CHAIN || tie_rule == MCGEN_TIE_CHUNK_ORDER) sb = mg::chain_scratch_bytes((long long)nx * nz);
    if ((e = scratch.alloc(sb))) return cuda_code(e);
    rc = mg::launch_quart_grid(w->desc, w->d_tree, (const MgLattice *)state.p, qx0, qz0, nx, nz, qy, tie_rule, d_out,
                               scratch.p, st);
    return rc ? cuda_code((cudaError_t)rc) : MCGEN_OK;
}

MCGEN_API long long mcgen_gb300_launch_count(void) { return mg::launch_count(); }
MCGEN_API int mcgen_gb300_profile(int enable) { return mg::prof_enable(enable) ? MCGEN_E_INTERNAL : MCGEN_OK; }
MCGEN_API int mcgen_gb300_profile_read(int kernel, const char **name, double *total_ms, long long *launches) {
    if (name) *name = mg::kernel_name(kernel);
    return mg::prof_read(kernel, total_ms, launches) ? MCGEN_E_ARG : MCGEN_OK;
}
MCGEN_API const char *mcgen_gb300_last_error(void) { return t_last_error.c_str(); }

MCGEN_API int mcgen_gb300_pipe_rate(int pipe, double *gops) {
    if (!gops) return MCGEN_E_ARG;
    std::lock_guard<std::mutex> lk(g_lock);
    if (!device_ready_locked()) return MCGEN_E_UNSUPPORTED;
    int rc = mg::pipe_rate(pipe, gops);
    return rc ? cuda_code((cudaError_t)rc) : MCGEN_OK;
}

/* Self-test: two independent device paths must agree -- the quart-grid kernel (shared-memory lattices) and
 * the seeds x points kernel (lattices through L1, separate setup launch) -- on npoints cells of every
 * dimension and preset of the version, for two seeds. */
MCGEN_API int mcgen_gpu_selftest(McGen *g, int npoints, char *report, size_t replen) {
    if (!g) return MCGEN_E_ARG;
    if (npoints <= 0) npoints = 384;
    int side = 1;
    while (side * side < npoints) side++;
    std::string rep;
    int bad_total = 0, rc_all = MCGEN_OK;
    const int64_t seeds[2] = {12345, -3141592653589793LL};
    for (int d = 0; d < 3 && rc_all == MCGEN_OK; d++)
        for (int p = 0; p < mg::preset_count(d) && rc_all == MCGEN_OK; p++)
            for (int s = 0; s < 2 && rc_all == MCGEN_OK; s++) {
                McSeeds sd = mcgen_seeds_unified(seeds[s]);
                McWorld *w = nullptr;
                char err[256];
                int rc = mcgen_world_new(g, dim_name(d), mg::preset_name(d, p), &sd, nullptr, 0, &w, err, sizeof err);
                if (rc) { rc_all = rc; rep += std::string("world: ") + err + "\n"; break; }
                std::vector<uint8_t> a((size_t)side * side), b((size_t)side * side);
                std::vector<int32_t> pts;
                for (int iz = 0; iz < side; iz++)
                    for (int ix = 0; ix < side; ix++) { pts.push_back(ix * 37 - 700); pts.push_back(16); pts.push_back(iz * 41 - 900); }
                /* the sampled cells lie on a lattice of stride (37, 41): take them from grid rows */
                std::vector<uint8_t> row((size_t)side * 37);
                int bad = 0;
                rc = MCGEN_OK;
                for (int iz = 0; iz < side && rc == MCGEN_OK; iz++) {
                    rc = mcgen_gb300_quart_grid(w, -700, iz * 41 - 900, side * 37, 1, 16, MCGEN_TIE_ENGINE, row.data());
                    for (int ix = 0; ix < side && rc == MCGEN_OK; ix++) a[(size_t)iz * side + ix] = row[(size_t)ix * 37];
                }
                if (rc == MCGEN_OK) rc = mcgen_gb300_seed_points(w, &seeds[s], 1, pts.data(), side * side, b.data(), nullptr);
                if (rc) rc_all = rc;
                for (size_t i = 0; i < a.size(); i++) bad += a[i] != b[i];
                bad_total += bad;
                char line[160];
                snprintf(line, sizeof line, "%s %s seed %lld: %d/%d mismatches\n", dim_name(d), mg::preset_name(d, p),
                         (long long)seeds[s], bad, side * side);
                rep += line;
                mcgen_world_free(w);
            }
    {
        std::lock_guard<std::mutex> lk(g_lock);
        g_selftest = rc_all ? "error" : (bad_total ? "mismatch" : "ok");
        if (rc_all == MCGEN_OK) (bad_total ? g_worlds_failed : g_worlds_ok)++;
    }
    if (report && replen) snprintf(report, replen, "%s", rep.c_str());
    if (rc_all) return rc_all;
    return bad_total ? MCGEN_E_INTERNAL : MCGEN_OK;
}

}  // extern "C"
