"""Build recipe of the oracle (test infrastructure): g++ -O2 -ffp-contract=off
(no fast-math, no FMA contraction) so every float expression is evaluated as
the written sequence of IEEE binary32 operations.  Output: oracle/_build/liboracle.so

The synthetic-scene generator (seeded terrain, materials, orbit cameras, the
PCG32 seed stream; no reference counterpart) is compiled into the oracle as
well, from the library's own source file with its entry points renamed
vrg_* -> orc_*, so that a CPU-only run (the benchmark's reference arm) builds
the very same inputs without loading the CUDA library.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_build", "liboracle.so")
TERRAIN = os.path.join(HERE, "..", "vulkan-voxel-restir-gi_gb300", "csrc", "terrain.cpp")


def build():
    os.makedirs(os.path.dirname(OUT), exist_ok=True)
    tmp = OUT + ".tmp"
    renames = [f"-D{n}=orc_{n[4:]}" for n in
               ("vrg_terrain_materials", "vrg_terrain_generate", "vrg_orbit_camera", "vrg_pcg32_next")]
    cmd = ["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fno-math-errno", "-fopenmp", "-fPIC", "-shared",
           "-Wall", "-o", tmp, os.path.join(HERE, "vrg_oracle.cpp")] + renames + [TERRAIN]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stdout + r.stderr)
    os.replace(tmp, OUT)
    return OUT


if __name__ == "__main__":
    print(build())
