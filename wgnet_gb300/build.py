"""Build the CUDA library `wgnet_gb300/_native/libwgnet_gb300.so` for sm_103a with nvcc.

Every `.cu` file under `csrc/` is compiled in parallel into `_build/` and linked into one shared
library (CUDA runtime linked statically). Rebuilds only what is older than its sources.

    python -m wgnet_gb300.build            # build if needed
    python -m wgnet_gb300.build --force    # rebuild everything
"""

from __future__ import annotations

import argparse
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
OUT_DIR = PKG / "_native"
LIB = OUT_DIR / "libwgnet_gb300.so"
INCLUDE = ROOT / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# -fmad=false: no contraction of a*b+c, so every f32 operation rounds as in the reference.
# -Xcompiler -ffp-contract=off: the same for host code (g++ contracts by default on aarch64), so the
# host-side wavelet and C-PML profiles are identical on x86_64 and aarch64.
NVCC_FLAGS = ["-O3", "-std=c++17", "-fmad=false", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
              "-Xcompiler", "-ffp-contract=off", "--expt-relaxed-constexpr"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build wgnet_gb300")


def _headers() -> list[Path]:
    return sorted(list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + list(INCLUDE.glob("*.h")))


def build(force: bool = False, verbose: bool = False) -> Path:
    sources = sorted(CSRC.glob("*.cu"))
    BUILD.mkdir(exist_ok=True)
    OUT_DIR.mkdir(exist_ok=True)
    stamp = BUILD / "flags.txt"
    flags = " ".join([*ARCH, *NVCC_FLAGS, os.uname().machine])
    if not stamp.exists() or stamp.read_text() != flags:
        force = True
        stamp.write_text(flags)
    hdr_mtime = max((h.stat().st_mtime for h in _headers()), default=0.0)
    jobs = []
    objs = []
    exe = nvcc()
    for src in sources:
        obj = BUILD / (src.stem + ".o")
        objs.append(obj)
        if not force and obj.exists() and obj.stat().st_mtime >= max(src.stat().st_mtime, hdr_mtime):
            continue
        cmd = [exe, *ARCH, *NVCC_FLAGS, f"-I{INCLUDE}", f"-I{CSRC}", "-c", str(src), "-o", str(obj)]
        if verbose:
            print(" ".join(cmd), flush=True)
        jobs.append((src, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)))
    failed = []
    for src, proc in jobs:
        out, _ = proc.communicate()
        if proc.returncode != 0:
            failed.append((src, out))
        elif verbose and out.strip():
            print(out, flush=True)
    if failed:
        msg = "\n".join(f"--- {s.name}\n{o}" for s, o in failed)
        raise RuntimeError(f"nvcc failed for {len(failed)} file(s):\n{msg}")
    newest = max(o.stat().st_mtime for o in objs)
    if force or jobs or not LIB.exists() or LIB.stat().st_mtime < newest:
        tmp = LIB.with_suffix(".so.tmp")
        cmd = [exe, *ARCH, "-shared", "-o", str(tmp), *map(str, objs)]
        res = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"link failed:\n{res.stdout}")
        os.replace(tmp, LIB)
    return LIB


def main(argv: list[str] | None = None) -> int:
    ap = argparse.ArgumentParser(description=__doc__)
    ap.add_argument("--force", action="store_true")
    ap.add_argument("-v", "--verbose", action="store_true")
    args = ap.parse_args(argv)
    path = build(force=args.force, verbose=args.verbose)
    print(path)
    return 0


if __name__ == "__main__":
    sys.exit(main())
