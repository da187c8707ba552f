"""ORACLE -- test infrastructure only.  Times the unmodified reference
renderer (oracle/_ref/pathtracer, built by `make -C oracle ref` against the
Embree-API shim; x86 only) and the C port (oracle/oc_render.c, the CPU
baseline bench.py reports on the GPU host) on the same benchmark frame and the
same host cores, to show how the port compares with the reference itself.

    python oracle/time_reference.py [spp]     (default 8)
"""
import importlib
import os
import re
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path[:0] = [ROOT, HERE]


def main() -> None:
    spp = int(sys.argv[1]) if len(sys.argv) > 1 else 8
    scenes = importlib.import_module("openmaterial-validation_gb300.scenes")
    import bench
    import oracle

    sc = scenes.scene_c2(1920, 1080, spp)
    d = tempfile.mkdtemp()
    out = scenes.write_gltf(sc, d)
    exe = os.path.join(HERE, "_ref", "pathtracer")
    threads = os.cpu_count() or 1
    r = subprocess.run([exe, *out["flags"], "-C", str(threads), "-o", os.path.join(d, "out.png")],
                       capture_output=True, text=True, cwd=d, check=True)
    dur = float(re.search(r"Duration: ([0-9.]+) seconds", r.stdout).group(1))
    paths = 1920 * 1080 * spp
    print(f"reference (shim BVH): {paths / dur / 1e6:.2f} Mpaths/s, {threads} threads, {dur:.1f} s")
    oracle.build()
    v, _, t, rows, dt = bench.cpu_reference(oracle, sc, spp, target_s=30.0)
    print(f"port:                 {v:.2f} Mpaths/s, {t} threads, {rows} rows in {dt:.1f} s")


if __name__ == "__main__":
    main()
