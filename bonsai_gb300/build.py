"""Builds libbonsai_gpu.so in-tree (bonsai_gb300/lib/) for sm_103a.

CUDA sources: nvcc -gencode arch=compute_103a,code=sm_103a -O3 -lineinfo, with -fmad=false for
the units that hold traversal, the reference-compatible (REF_COMPAT) kernels and the per-thread
integrators: there every float operation rounds as written (the reference is Rust f32, which never
contracts a*b+c), and kernels use fmaf() where a fused product is intended.  The PBRT-mode shading
units and the guiding network's kernels (FUSED_SOURCES) let nvcc contract products into fused
multiply-adds; the triangle test and the error-free products they share with traversal, and the
lobe concentration that inference and shading both derive from a stored mixture, are written with
explicitly rounded intrinsics, so they round the same in every unit.
Host sources: g++ -O2 -ffp-contract=off.  Translation units compile in parallel.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
OBJ = PKG / "_build"
LIB = PKG / "lib" / "libbonsai_gpu.so"
CUDA = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

CU_SOURCES = ["bg_kernels.cu", "bg_shade_plain.cu", "bg_shade_aux.cu", "bg_shade_guided_full.cu", "bg_shade_shapes.cu",
              "bg_noalloc.cu",
              "bg_guide.cu",
              "bg_integrators.cu", "bg_integrators_pbrt.cu", "bg_tree_wave.cu",
              "bg_tree_shade_w.cu", "bg_tree_shade_d.cu"]
CPP_SOURCES = ["bg_api.cpp", "bg_bvh.cpp", "bg_guide_api.cpp", "bg_io.cpp"]
# PBRT-mode shade launches (wavefront, guided, batch, Whitted / direct-lighting tree wavefront) and
# the guiding network
FUSED_SOURCES = {"bg_shade_plain.cu", "bg_shade_aux.cu", "bg_shade_guided_full.cu", "bg_shade_shapes.cu",
                 "bg_tree_shade_w.cu", "bg_tree_shade_d.cu", "bg_guide.cu"}


def _nvcc() -> str:
    p = CUDA / "bin" / "nvcc"
    return str(p) if p.exists() else (shutil.which("nvcc") or "nvcc")


def commands() -> tuple[list[list[str]], list[str]]:
    OBJ.mkdir(exist_ok=True)
    LIB.parent.mkdir(exist_ok=True)
    cmds, objs = [], []
    for src in CU_SOURCES:
        o = str(OBJ / (Path(src).stem + ".o"))
        defines = os.environ.get("BONSAI_NVCC_DEFINES", "").split()  # -DNAME=VALUE traversal variants
        fmad = "-fmad=true" if src in FUSED_SOURCES else "-fmad=false"
        cmds.append([_nvcc(), *ARCH, "-O3", "-lineinfo", fmad, "-std=c++17", "-Xcompiler", "-fPIC",
                     "-Xptxas", "-warn-spills", *defines, "-c", str(CSRC / src), "-o", o])
        objs.append(o)
    for src in CPP_SOURCES:
        o = str(OBJ / (Path(src).stem + ".o"))
        cmds.append(["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-Wall",
                     f"-I{CUDA / 'include'}", "-c", str(CSRC / src), "-o", o])
        objs.append(o)
    return cmds, objs


def build(verbose: bool = False) -> Path:
    cmds, objs = commands()
    procs = [subprocess.Popen(c, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True) for c in cmds]
    failed = []
    for c, p in zip(cmds, procs):
        out, _ = p.communicate()
        if verbose and out.strip():
            print(out, file=sys.stderr)
        if p.returncode != 0:
            failed.append((c, out))
    if failed:
        msg = "\n".join(" ".join(c) + "\n" + out for c, out in failed)
        raise RuntimeError(f"compilation failed:\n{msg}")
    link = [_nvcc(), *ARCH, "-shared", "-o", str(LIB), *objs, "-lpthread"]
    r = subprocess.run(link, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n" + " ".join(link) + "\n" + r.stdout)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
