"""Build recipe of oracle/_ref/libsph_ref.so: the reference's own plain-step
code (its device functions and kernels, compiled for the host) behind the
harness oracle/ref_harness.cpp.  Test infrastructure only.

The recipe reads the reference checkout (argument or $SPH_REFERENCE_DIR,
default /root/reference): from CUDASPHNEW/particle_simulation.h the VD/SD
enums and SimulationParameters, and from CUDASPHNEW/particle_simulation.cu
the definitions of the functions listed below, copied as they are, in that
order, into oracle/_ref/ref_types.inc and oracle/_ref/ref_funcs.inc.  Those
files and the library are build outputs (oracle/_ref/ is not committed).
Where the checkout is absent, files extracted earlier are compiled as they
are; with neither, the recipe does nothing.

    python oracle/build_ref.py [<reference checkout>]
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
LIB_PATH = os.path.join(OUT, "libsph_ref.so")

# device helpers first (the kernels call them), then the kernels of the step
FUNCTIONS = [
    "compute_grid_coordinate", "compute_hash_from_grid_coordinate", "norm", "normalize", "compute_distance",
    "compute_squared_distance", "dot_product", "compute_particle_density_cell",
    "compute_viscosity_pressure_forces_and_ifsurf_cell",
    "compute_particle_hash", "compute_particle_density_pressure", "compute_particle_acceleration_ifsurf",
    "integrate_euler", "collision_handling",
]


def reference_dir(arg: str | None = None) -> str:
    return os.path.join(arg or os.environ.get("SPH_REFERENCE_DIR", "/root/reference"), "CUDASPHNEW")


def definition(src: str, name: str) -> str:
    """The text of the definition of `name` (from the line that starts it to
    its closing brace); declarations (ending in ';' before any '{') are skipped."""
    lines = src.splitlines(keepends=True)
    for k, line in enumerate(lines):
        head = line.split("(")[0].split()
        if not head or head[-1] != name or not line.lstrip().startswith(("__device__", "__global__")):
            continue
        rest = "".join(lines[k:])
        brace, semi = rest.find("{"), rest.find(";")
        if brace < 0 or (0 <= semi < brace):
            continue  # a declaration
        depth, i = 0, brace
        while True:
            c = rest[i]
            if c == "{":
                depth += 1
            elif c == "}":
                depth -= 1
                if depth == 0:
                    return rest[: i + 1] + "\n"
            i += 1
    raise ValueError(f"no definition of {name}")


def types(header: str) -> str:
    """From `enum ParticleVertexDataIdx` to the end of `struct SimulationParameters`."""
    a = header.index("enum ParticleVertexDataIdx")
    b = header.index("struct SimulationParameters")
    c = header.index("};", b) + 2
    return header[a:c] + "\n"


def build(ref: str | None = None, force: bool = False) -> str | None:
    """Extracts the reference's functions (where the checkout is present) and
    compiles the harness.  Without the checkout, files extracted earlier in
    oracle/_ref/ (they travel with a copy of the working tree) are compiled
    as they are; with neither, nothing is built (None)."""
    d = reference_dir(ref)
    cu, h = os.path.join(d, "particle_simulation.cu"), os.path.join(d, "particle_simulation.h")
    types_inc, funcs_inc = os.path.join(OUT, "ref_types.inc"), os.path.join(OUT, "ref_funcs.inc")
    have_checkout = os.path.exists(cu) and os.path.exists(h)
    if not have_checkout and not (os.path.exists(types_inc) and os.path.exists(funcs_inc)):
        return None
    harness = os.path.join(HERE, "ref_harness.cpp")
    if (not force and os.path.exists(LIB_PATH)
            and os.path.getmtime(LIB_PATH) >= max(os.path.getmtime(harness), os.path.getmtime(__file__))):
        return LIB_PATH
    os.makedirs(OUT, exist_ok=True)
    if have_checkout:
        src = open(cu, encoding="latin-1").read()
        with open(types_inc, "w") as f:
            f.write(types(open(h, encoding="latin-1").read()))
        with open(funcs_inc, "w") as f:
            for name in FUNCTIONS:
                f.write(definition(src, name))
    tmp = LIB_PATH + ".tmp"
    cmd = ["g++", "-std=c++17", "-O2", "-fopenmp", "-shared", "-fPIC", "-ffp-contract=off",
           "-ftrivial-auto-var-init=zero", "-w", "-I", HERE, harness, "-o", tmp]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build of the reference harness failed:\n{r.stderr}")
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    print(build(sys.argv[1] if len(sys.argv) > 1 else None, force=True))
