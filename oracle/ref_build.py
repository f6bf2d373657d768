"""Build the reference's own engine into oracle/_ref/ — TEST INFRASTRUCTURE ONLY.

Recipe for the two reference builds this repository measures against; it
reads the reference's sources where they lie and writes only into
``oracle/_ref/`` (git-ignored).  It does not run the reference's build
system (``torch.utils.cpp_extension.load`` in qmb/hamiltonian.py:58-65); it
calls the compilers directly with the flags that load() would pass.

* ``cpu``: ``qmb/_hamiltonian.cpp`` (operator schemas) + ``qmb/_hamiltonian_cpu.cpp``
  compiled by g++ with the reference's flags (``-O3 -ffast-math
  -march=native -std=c++20 -DN_QUBYTES=<nq> -DPARTICLE_CUT=<pc>``) into a
  shared library that ``torch.ops.load_library`` loads, registering
  ``torch.ops.qmb_hamiltonian_<nq>_<pc>.apply_within/find_relative`` on the
  CPU.  Host code for this machine only (x86): used to time the reference's
  CPU engine beside the oracle port on the same cores.
* ``cuda``: ``qmb/_hamiltonian_cuda.cu`` compiled by nvcc for sm_103a
  (``-O3 --use_fast_math -std=c++20`` plus the macros torch's extension
  build adds) into a device-code-only cubin, with the mangled names of its
  kernels (read from ptxas's ``-v`` report) in a JSON file beside it.  A
  cubin holds no host code, so it loads on the GPU host through the CUDA
  driver API (oracle/ref_cuda.py) although the reference's sources are not
  there.

Usage: ``python oracle/ref_build.py [--nq 4] [--pc 1] [cpu|cuda ...]``.
"""

from __future__ import annotations

import argparse
import json
import os
import re
import shutil
import subprocess
import sys
import sysconfig

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
REFERENCE = "/root/reference/qmb"


def available() -> bool:
    return os.path.isdir(REFERENCE)


def _torch_flags() -> tuple[list[str], list[str], str]:
    import torch.utils.cpp_extension as ext

    includes = [f"-I{p}" for p in ext.include_paths()] + [f"-I{sysconfig.get_paths()['include']}"]
    nvcc_common = list(ext.COMMON_NVCC_FLAGS)
    libdir = os.path.join(os.path.dirname(ext.__file__), "..", "lib")
    return includes, nvcc_common, os.path.abspath(libdir)


def cpu_library(nq: int, pc: int) -> str:
    return os.path.join(OUT, f"libqmb_ref_cpu_{nq}_{pc}.so")


def cuda_cubin(nq: int, pc: int) -> str:
    return os.path.join(OUT, f"ref_cuda_{nq}_{pc}.cubin")


def build_cpu(nq: int, pc: int) -> str:
    out = cpu_library(nq, pc)
    if os.path.exists(out):
        return out
    includes, _, libdir = _torch_flags()
    os.makedirs(OUT, exist_ok=True)
    name = f"qmb_hamiltonian_{nq}_{pc}"
    cmd = [os.environ.get("CXX", "g++"), "-shared", "-fPIC", "-O3", "-ffast-math", "-march=native", "-std=c++20",
           f"-DN_QUBYTES={nq}", f"-DPARTICLE_CUT={pc}", f"-DTORCH_EXTENSION_NAME={name}",
           "-DTORCH_API_INCLUDE_EXTENSION_H", *includes,
           os.path.join(REFERENCE, "_hamiltonian.cpp"), os.path.join(REFERENCE, "_hamiltonian_cpu.cpp"),
           f"-L{libdir}", "-lc10", "-ltorch", "-ltorch_cpu", "-ltorch_python", f"-Wl,-rpath,{libdir}",
           "-o", out + ".tmp"]
    subprocess.run(cmd, check=True)
    os.replace(out + ".tmp", out)
    return out


def build_cuda(nq: int, pc: int) -> str:
    out = cuda_cubin(nq, pc)
    meta = out[:-len(".cubin")] + ".json"
    if os.path.exists(out) and os.path.exists(meta):
        return out
    includes, nvcc_common, _ = _torch_flags()
    os.makedirs(OUT, exist_ok=True)
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    name = f"qmb_hamiltonian_{nq}_{pc}"
    cmd = [nvcc, "-cubin", "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "--use_fast_math", "-std=c++20",
           f"-DN_QUBYTES={nq}", f"-DPARTICLE_CUT={pc}", *nvcc_common, "-DTORCH_API_INCLUDE_EXTENSION_H",
           f"-DTORCH_EXTENSION_NAME={name}", *includes, "-Xptxas", "-v",
           os.path.join(REFERENCE, "_hamiltonian_cuda.cu"), "-o", out + ".tmp"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed on the reference CUDA file:\n{res.stderr[-4000:]}")
    entries = re.findall(r"Compiling entry function '([^']+)'", res.stdout + res.stderr)
    kernels = {}
    for short in ("apply_within_kernel_interface", "find_relative_kernel_interface", "diagonal_term_kernel_interface",
                  "single_relative_kernel_interface"):
        hits = [e for e in entries if short in e]
        if hits:
            kernels[short] = hits[0]
    os.replace(out + ".tmp", out)
    with open(meta, "w") as f:
        json.dump({"n_qubytes": nq, "particle_cut": pc, "kernels": kernels,
                   "source": "qmb/_hamiltonian_cuda.cu", "flags": cmd[1:cmd.index("-Xptxas")]}, f, indent=1)
    return out


def main(argv=None) -> int:
    parser = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    parser.add_argument("what", nargs="*", default=["cpu", "cuda"])
    parser.add_argument("--nq", type=int, default=4)
    parser.add_argument("--pc", type=int, default=1)
    args = parser.parse_args(argv)
    if not available():
        print("reference sources not present; nothing built", file=sys.stderr)
        return 0
    for what in args.what:
        path = build_cpu(args.nq, args.pc) if what == "cpu" else build_cuda(args.nq, args.pc)
        print(path)
    return 0


if __name__ == "__main__":
    sys.exit(main())
