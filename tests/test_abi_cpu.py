"""C-ABI host-side tests (CPU only, no GPU compute).

The library must build, load, and export every symbol include/*.h declares; host-side logic (data loading,
argument checks, names, error codes) is exercised without launching a kernel.
"""
import ctypes as C
import os
import re

import numpy as np
import pytest

import __graft_entry__ as ge

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="session")
def mg():
    ge._build_module().build()
    m = ge.package()
    m.load()
    return m


def declared_symbols():
    names = []
    for h in ("mcgen.h", "mcgen_gb300.h"):
        src = open(os.path.join(REPO, "include", h)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names += re.findall(r"MCGEN_API\s+[^;(]*?\b(mcgen_\w+)\s*\(", src)
    return sorted(set(names))


def test_exports_every_declared_symbol(mg):
    lib = C.CDLL(mg.LIB_PATH)
    names = declared_symbols()
    assert len(names) >= 50
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_links_as_libmcgen(mg, tmp_path):
    """A C caller of the reference library links with -lmcgen unchanged: build.py provides libmcgen.so,
    and a program built against include/mcgen.h alone runs against it (host calls only, no device)."""
    import shutil
    import subprocess

    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    src = tmp_path / "caller.c"
    src.write_text('#include <stdio.h>\n#include "mcgen.h"\n'
                   'int main(void) { printf("%d %s\\n", mcgen_abi_version(), mcgen_version()); return 0; }\n')
    lib_dir = os.path.dirname(mg.LIB_PATH)
    assert os.path.exists(os.path.join(lib_dir, "libmcgen.so"))
    exe = tmp_path / "caller"
    subprocess.run([cc, str(src), "-I", os.path.join(REPO, "include"), "-L", lib_dir, "-lmcgen", "-o", str(exe)],
                   check=True, capture_output=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, env={**os.environ, "LD_LIBRARY_PATH": lib_dir})
    assert r.returncode == 0, r.stderr
    assert r.stdout.startswith("1 ") and "abi 1" in r.stdout


def test_version(mg):
    L = mg.load()
    assert L.mcgen_abi_version() == 1
    assert b"abi 1" in L.mcgen_version()


def test_open_errors(mg):
    with pytest.raises(mg.McError) as e:
        mg.Generator.open(ge.data_root(), "25.9")
    assert e.value.code == mg.MCGEN_E_VERSION
    with pytest.raises(mg.McError) as e:
        mg.Generator.open("/nonexistent-data-root", "26.3")
    assert e.value.code == mg.MCGEN_E_IO


@pytest.mark.parametrize("version", ["26.1", "26.2", "26.3", "26.4-snapshot-2"])
def test_names_and_presets(mg, version):
    g = mg.Generator.open(ge.data_root(), version)
    assert g.dimensions() == ["minecraft:overworld", "minecraft:the_nether", "minecraft:the_end"]
    assert g.presets("minecraft:overworld") == ["normal", "amplified", "large_biomes"]
    assert g.presets("minecraft:the_nether") == ["normal"]
    names = g.biome_names()
    assert len(names) == 67 and names[0] == "minecraft:badlands" and names[41] == "minecraft:plains"
    L = mg.load()
    assert L.mcgen_block_state_count(g._h) == 0 and L.mcgen_tweak_count(g._h) == 0


def test_world_new_errors(mg):
    g = mg.Generator.open(ge.data_root(), "26.3")
    with pytest.raises(mg.McError) as e:
        g.world("minecraft:overworld_caves", "normal", 1)
    assert e.value.code == mg.MCGEN_E_ARG
    with pytest.raises(mg.McError) as e:
        g.world("minecraft:the_nether", "amplified", 1)
    assert e.value.code == mg.MCGEN_E_ARG
    w = g.world("minecraft:overworld", "large_biomes", 7)
    assert (w.min_y, w.height, w.sea_level) == (-64, 384, 63)
    n = g.world("minecraft:the_nether", None, 7)
    assert (n.min_y, n.height, n.sea_level) == (0, 256, 32)


def test_spline_nesting_limit(mg, tmp_path):
    """An offset spline that nests deeper than the device evaluator's stack (six multipoint levels; every
    shipped table nests four) is refused with MCGEN_E_DATA when the world is built, and six levels are
    accepted."""
    import shutil

    def spline(levels: int) -> str:
        s = "C 0.25"
        for _ in range(levels):
            s = f"S 0 1 0.0 0.0 {s}"
        return s

    for levels, ok in ((6, True), (7, False)):
        root = tmp_path / f"root{levels}"
        shutil.copytree(os.path.join(ge.data_root(), "data"), root / "data")
        f = root / "data" / "climate-26.3.txt"
        lines = [f"offset_spline overworld {spline(levels)}" if ln.startswith("offset_spline overworld ") else ln
                 for ln in f.read_text().splitlines()]
        f.write_text("\n".join(lines) + "\n")
        g = mg.Generator.open(str(root), "26.3")
        if ok:
            g.world("minecraft:overworld", "normal", 1)
        else:
            with pytest.raises(mg.McError) as e:
                g.world("minecraft:overworld", "normal", 1)
            assert e.value.code == mg.MCGEN_E_DATA


def test_world_info(mg):
    g = mg.Generator.open(ge.data_root(), "26.1")
    w = g.world("overworld", "normal", -42)
    v, d, s, f = C.c_int(), C.c_int(), C.c_int64(), C.c_int()
    assert mg.load().mcgen_gb300_world_info(w.handle, C.byref(v), C.byref(d), C.byref(s), C.byref(f)) == 0
    assert (v.value, d.value, s.value, f.value) == (0, 0, -42, 0)


def test_no_cpu_path(mg):
    """Biomes are computed on the GPU only: the CPU entry points refuse loudly."""
    g = mg.Generator.open(ge.data_root(), "26.3")
    w = g.world("minecraft:overworld", "normal", 1)
    L = mg.load()
    buf = (C.c_uint8 * 4)()
    assert L.mcgen_biome_grid_cpu(w.handle, 0, 0, 2, 2, 4, 64, C.cast(buf, C.c_void_p)) == mg.MCGEN_E_UNSUPPORTED
    assert L.mcgen_gpu_set_compute(mg.MCGEN_COMPUTE_CPU, -1) == mg.MCGEN_E_UNSUPPORTED
    out = C.c_void_p()
    assert L.mcgen_generate_region(w.handle, 0, 0, 1, 1, 1, 0, None, None, C.byref(out), None, 0) == mg.MCGEN_E_UNSUPPORTED


def test_argument_checks(mg):
    g = mg.Generator.open(ge.data_root(), "26.3")
    w = g.world("minecraft:overworld", "normal", 1)
    L = mg.load()
    buf = (C.c_uint8 * 4)()
    p = C.cast(buf, C.c_void_p)
    assert L.mcgen_biome_grid(w.handle, 0, 0, 0, 2, 4, 64, p) == mg.MCGEN_E_ARG
    assert L.mcgen_biome_grid(w.handle, 0, 0, 2, 2, 0, 64, p) == mg.MCGEN_E_ARG
    assert L.mcgen_biome_grid(None, 0, 0, 2, 2, 4, 64, p) == mg.MCGEN_E_ARG
    assert L.mcgen_biome_grid(w.handle, 0, 0, 2, 2, 4, 64, None) == mg.MCGEN_E_ARG
    assert L.mcgen_gb300_quart_grid(w.handle, 0, 0, 2, 2, 16, 7, p) == mg.MCGEN_E_ARG
    assert L.mcgen_biome_at(None, 0, 0, 0) == -1


@pytest.mark.skipif(ge.package().device_count() > 0 if os.path.exists(ge.package().LIB_PATH) else False,
                    reason="a CUDA device is present")
def test_no_device_fails_loudly(mg):
    g = mg.Generator.open(ge.data_root(), "26.3")
    w = g.world("minecraft:overworld", "normal", 1)
    with pytest.raises(mg.McError) as e:
        w.biome_grid(0, 0, 4, 4, 4, 64)
    assert e.value.code == mg.MCGEN_E_UNSUPPORTED
    assert w.biome_at(0, 64, 0) == -1
    ok, status = mg.gpu_status()
    assert not ok and "unavailable" in status


def test_plan_and_search_argument_checks(mg):
    """Argument checks of the batched and search entry points come before any device work."""
    g = mg.Generator.open(ge.data_root(), "26.3")
    w = g.world("minecraft:overworld", "normal", 1)
    L = mg.load()
    rq = (mg.McGb300Request * 2)(mg.McGb300Request(w.handle, 5, 0, 0, 4, 4, 16),
                                  mg.McGb300Request(w.handle, 6, 0, 0, 0, 4, 16))
    h = C.c_void_p()
    assert L.mcgen_gb300_plan_new(rq, 2, 0, C.byref(h)) == mg.MCGEN_E_ARG        # an empty region
    assert L.mcgen_gb300_plan_new(rq, 1, 1, C.byref(h)) == mg.MCGEN_E_ARG        # GRID_CHAIN is not a batch rule
    assert L.mcgen_gb300_plan_new(None, 1, 0, C.byref(h)) == mg.MCGEN_E_ARG
    obs = mg.make_obs([(0, 16, 0, [1])])
    found = (C.c_int64 * 4)()
    reached = (C.c_uint64 * 65)()
    nf = C.c_uint32()

    def search(o, n_obs, kind=1, lst=None, n=0):
        return L.mcgen_gb300_search(w.handle, kind, lst, C.c_uint64(0), C.c_uint64(n),
                                    o.ctypes.data if o is not None else None, n_obs, 1, found, 4, C.byref(nf), reached, None)

    assert search(obs, 0) == mg.MCGEN_E_ARG                                       # no observation
    assert search(obs, 65) == mg.MCGEN_E_ARG                                      # more than 64
    assert search(None, 1) == mg.MCGEN_E_ARG
    assert search(obs, 1, kind=3) == mg.MCGEN_E_ARG                               # unknown source
    assert search(obs, 1, kind=0, lst=None, n=10) == mg.MCGEN_E_ARG               # list source without a list
    bad = obs.copy()
    bad["flags"][0] = 13                                                          # End window half-width > 12
    assert search(bad, 1) == mg.MCGEN_E_ARG
    bad["flags"][0] = 0x200                                                       # unknown flag
    assert search(bad, 1) == mg.MCGEN_E_ARG
    assert L.mcgen_gb300_obs_end_radius(None, None) == -1


def test_request_packing(mg):
    """Request lists packed as numpy records are byte-identical to McGb300Request arrays (signed and unsigned
    64-bit seeds, one world or one per request), and out-of-range fields are rejected on the host."""
    g = mg.Generator.open(ge.data_root(), "26.3")
    w1 = g.world("minecraft:overworld", "normal", 1)
    w2 = g.world("minecraft:the_end", "normal", 1)
    seeds = [-(2**63), 2**63 - 1, 2**63 + 7, 0, 12345]
    reqs = [(w1 if i % 2 else w2, s, i - 3, 5 * i, 16 + i, 9, 16 - i) for i, s in enumerate(seeds)]
    ref = (mg.McGb300Request * len(reqs))()
    for i, (w, s, qx, qz, nx, nz, qy) in enumerate(reqs):
        ref[i] = mg.McGb300Request(w.handle, s - 2**64 if s >= 2**63 else s, qx, qz, nx, nz, qy)
    rec, worlds = mg._pack_requests(reqs)
    assert rec.tobytes() == bytes(ref) and worlds == [r[0] for r in reqs]
    ra = mg.RequestArray([r[0] for r in reqs], np.array([s % 2**64 for s in seeds], np.uint64),
                         [r[2] for r in reqs], [r[3] for r in reqs], [r[4] for r in reqs], 9, [r[6] for r in reqs])
    assert ra.records.tobytes() == bytes(ref) and len(ra) == len(reqs)
    one = mg.RequestArray(w1, np.arange(4), 0, 0, 8, 8)
    assert (one.records["world"] == w1.handle.value).all() and (one.records["qy"] == 16).all()
    with pytest.raises(ValueError):
        mg._pack_requests([(w1, 1, 2**31, 0, 4, 4, 16)])
    with pytest.raises(ValueError):
        mg.RequestArray(w1, [1, 2], 0, [0, -2**31 - 1], 4, 4)
    with pytest.raises(ValueError):
        mg.RequestArray([w1], [1, 2], 0, 0, 4, 4)
