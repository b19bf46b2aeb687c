"""Build recipe for the CPU oracle (test infrastructure).

* ``oracle/liboracle.so``      the C++ restatement in oracle.cpp (always).
* ``oracle/_ref/libaxisref.so`` the reference's own header-only geometry code
  compiled unchanged from the reference checkout through the host shim in
  ``oracle/ref_shim`` plus the glue in ``ref_driver.cpp``; built only when the
  reference checkout exists (never on machines without it).
* ``oracle/_ref/libaxisref_fast.so`` the reference's regular/rectilinear
  fast-path sources (four files of src/solver/) compiled unchanged the same
  way, with ``ref_fast.cpp``; also only where the checkout exists.
* ``oracle/_ref/libaxisref_gen.so`` the reference's whole weight generator
  (src/solver/weight_generator.cpp and the solver sources it calls) compiled
  unchanged the same way, ArborX replaced by the exhaustive search of
  ``ref_shim/ArborX.hpp``, with ``ref_generate.cpp``; also only where the
  checkout exists.
* ``oracle/_ref/libaxisref_apply.so`` the reference's NaN-aware and masked
  applies (include/axis/solver/apply.hpp), weight-cache serializer
  (weight_cache.hpp) and conservation report (src/solver/conservation.cpp),
  compiled unchanged the same way, with ``ref_apply.cpp``; also only where
  the checkout exists.

Both use ``-O2 -ffp-contract=off`` so double expressions are evaluated as
written, like the reference's host build.
"""

from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
# The reference checkout: $AXGB_REFERENCE_ROOT, else a directory "reference"
# beside the repository.
REF_ROOT = os.environ.get("AXGB_REFERENCE_ROOT") or os.path.normpath(os.path.join(HERE, "..", "..", "reference"))
REF_INCLUDE = os.path.join(REF_ROOT, "libs", "axis", "include")
FLAGS = ["-std=c++20", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-fopenmp"]


def _needs(out: str, srcs: list[str]) -> bool:
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(s) > t for s in srcs)


def build_oracle(force: bool = False) -> str:
    src = os.path.join(HERE, "oracle.cpp")
    out = os.path.join(HERE, "liboracle.so")
    if force or _needs(out, [src]):
        subprocess.check_call(["g++", *FLAGS, src, "-o", out])
    return out


def build_ref(force: bool = False) -> str | None:
    if not os.path.isdir(REF_INCLUDE):
        return None
    src = os.path.join(HERE, "ref_driver.cpp")
    shim = os.path.join(HERE, "ref_shim")
    outdir = os.path.join(HERE, "_ref")
    os.makedirs(outdir, exist_ok=True)
    out = os.path.join(outdir, "libaxisref.so")
    deps = [src] + [os.path.join(shim, f) for f in ("Kokkos_Core.hpp", "mdspan/mdspan.hpp")]
    if force or _needs(out, deps):
        subprocess.check_call(["g++", *[f for f in FLAGS if f != "-fopenmp"], "-I", shim, "-I", REF_INCLUDE, src,
                               "-o", out])
    return out


REF_SRC = os.path.join(REF_ROOT, "libs", "axis", "src", "solver")
FAST_SOURCES = ["weight_generator_conservative_rect.cpp", "weight_generator_conservative_rect_nonuniform.cpp",
                "weight_generator_bilinear_rect.cpp", "weight_generator_bilinear_rect_nonuniform.cpp"]


def build_ref_fast(force: bool = False) -> str | None:
    """oracle/_ref/libaxisref_fast.so: the reference's regular/rectilinear
    fast-path sources compiled unchanged where they lie, with ref_fast.cpp."""
    if not os.path.isdir(REF_SRC):
        return None
    shim = os.path.join(HERE, "ref_shim")
    outdir = os.path.join(HERE, "_ref")
    os.makedirs(outdir, exist_ok=True)
    out = os.path.join(outdir, "libaxisref_fast.so")
    srcs = [os.path.join(HERE, "ref_fast.cpp")] + [os.path.join(REF_SRC, f) for f in FAST_SOURCES]
    deps = srcs + [os.path.join(shim, f) for f in ("Kokkos_Core.hpp", "KokkosSparse_CrsMatrix.hpp")]
    if force or _needs(out, deps):
        subprocess.check_call(["g++", *[f for f in FLAGS if f != "-fopenmp"], "-I", shim, "-I", REF_INCLUDE, *srcs,
                               "-o", out])
    return out


GEN_SOURCES = ["weight_generator.cpp", *FAST_SOURCES, "gradient_reconstructor.cpp", "halo_pattern.cpp",
               "interpolation_matrix.cpp"]
SHIM_HEADERS = ["Kokkos_Core.hpp", "KokkosSparse_CrsMatrix.hpp", "KokkosSparse_spmv.hpp", "Kokkos_UnorderedMap.hpp",
                "ArborX.hpp"]


def build_ref_gen(force: bool = False) -> str | None:
    """oracle/_ref/libaxisref_gen.so: WeightGenerator::generate of the
    reference, compiled unchanged where its sources lie, with ref_generate.cpp."""
    if not os.path.isdir(REF_SRC):
        return None
    shim = os.path.join(HERE, "ref_shim")
    outdir = os.path.join(HERE, "_ref")
    os.makedirs(outdir, exist_ok=True)
    out = os.path.join(outdir, "libaxisref_gen.so")
    srcs = [os.path.join(HERE, "ref_generate.cpp")] + [os.path.join(REF_SRC, f) for f in GEN_SOURCES]
    deps = srcs + [os.path.join(shim, f) for f in SHIM_HEADERS]
    if force or _needs(out, deps):
        subprocess.check_call(["g++", *[f for f in FLAGS if f != "-fopenmp"], "-Wl,--no-undefined", "-I", shim,
                               "-I", REF_INCLUDE, *srcs, "-o", out])
    return out


def build_ref_apply(force: bool = False) -> str | None:
    """oracle/_ref/libaxisref_apply.so: nan_batch_apply and the masked apply
    of the reference's apply.hpp, its WeightCache::serialize and
    check_conservation (conservation.cpp), with ref_apply.cpp."""
    if not os.path.isdir(REF_SRC):
        return None
    shim = os.path.join(HERE, "ref_shim")
    outdir = os.path.join(HERE, "_ref")
    os.makedirs(outdir, exist_ok=True)
    out = os.path.join(outdir, "libaxisref_apply.so")
    srcs = [os.path.join(HERE, "ref_apply.cpp")] + [os.path.join(REF_SRC, f) for f in
                                                     ("halo_pattern.cpp", "interpolation_matrix.cpp",
                                                      "conservation.cpp")]
    solver_inc = os.path.join(REF_INCLUDE, "axis", "solver")
    deps = (srcs + [os.path.join(shim, f) for f in SHIM_HEADERS] +
            [os.path.join(solver_inc, f) for f in ("apply.hpp", "weight_cache.hpp")])
    if force or _needs(out, deps):
        subprocess.check_call(["g++", *[f for f in FLAGS if f != "-fopenmp"], "-Wl,--no-undefined", "-I", shim,
                               "-I", REF_INCLUDE, *srcs, "-o", out])
    return out


if __name__ == "__main__":
    force = "--force" in sys.argv
    print(build_oracle(force))
    print(build_ref(force))
    print(build_ref_fast(force))
    print(build_ref_gen(force))
    print(build_ref_apply(force))
