"""Copy the seed-independent game tables that a world is built from into the package's data root.

``mcgen_open(root, version)`` reads ``<root>/data/climate-<V>.txt`` (noise parameters, presets, depth
gradient, ridges-folded constants, offset spline) and ``<root>/data/params/<V>/{overworld,nether}.tsv``
(the multi-noise biome parameter lists), the same layout the reference engine loads
(engine/mc_data.h:84-183).  The tables are game data extracted from Minecraft by the reference
project; they are copied verbatim so the library can run where the reference tree is absent.  This is a
provenance script of the build container (like make_fixtures.py beside it), not part of the library.

Usage:  python tests/golden/sync_tables.py   (MCGEN_REFERENCE_ROOT: the reference source tree)
"""
import os
import shutil

SRC = os.path.join(os.environ.get("MCGEN_REFERENCE_ROOT", "/root/reference"), "data")
DST = os.path.join(os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__)))),
                   "mc-worldgen-seed-lab_gb300", "data")
VERSIONS = ["26.1", "26.2", "26.3", "26.4-snapshot-2"]

if __name__ == "__main__":
    for v in VERSIONS:
        shutil.copyfile(os.path.join(SRC, f"climate-{v}.txt"), os.path.join(DST, f"climate-{v}.txt"))
        os.makedirs(os.path.join(DST, "params", v), exist_ok=True)
        for f in ("overworld.tsv", "nether.tsv"):
            shutil.copyfile(os.path.join(SRC, "params", v, f), os.path.join(DST, "params", v, f))
    print("tables copied to", DST)
