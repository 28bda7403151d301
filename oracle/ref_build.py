"""Recipe: compile the reference's own CPU-runnable code into oracle/_ref/.

TEST INFRASTRUCTURE ONLY.  For each example model of the reference
(examples/<dir>/model.cuh) this builds ``oracle/_ref/libref_<name>.so`` from
the reference's sources where they lie (nothing is copied into this repo):

  * src/gpu_mcmc.cu up to (not including) ``void run_mcmc`` -- the kernels --
    is streamed through ``sed`` into ``g++ -x c++ -`` with the shim headers of
    oracle/ref_shim/ first on the include path (kernel qualifiers removed,
    curand replaced by injected streams) and the example's model.cuh found
    through ``-I``;
  * oracle/ref_driver.cpp supplies the launch loops of run_mcmc /
    run_calcmodchi2 / run_calcmodel.

Only this container has the reference tree; the outputs are used here to
generate the committed golden fixtures (tests/golden/make_golden.py).
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
SHIM = os.path.join(HERE, "ref_shim")
REF_ROOT = os.environ.get("CUDA_MCMC_REFERENCE", "/root/reference")

MODELS = {"sgra": "examples/sgra_model_fit",
          "rosenbrock": "examples/search_Rosenbrock",
          "solvsys": "examples/solvsys"}


def _host_has_fma() -> bool:
    try:
        with open("/proc/cpuinfo") as f:
            return " fma " in f.read()
    except OSError:
        return False


def available() -> bool:
    return os.path.isfile(os.path.join(REF_ROOT, "src", "gpu_mcmc.cu"))


def lib_path(name: str) -> str:
    return os.path.join(OUT, "libref_%s.so" % name)


def build(force: bool = False) -> list:
    if not available():
        return []
    os.makedirs(OUT, exist_ok=True)
    src = os.path.join(REF_ROOT, "src")
    # nvcc contracts a*b + c into fused multiply-adds by default (-fmad=true);
    # -ffp-contract=fast with FMA instructions gives the host build the same
    # single-rounding proposal step p + pstp*N(0,1) as the reference's GPU build.
    fma = ["-mfma"] if _host_has_fma() else []
    flags = ["-std=c++17", "-O2", "-fPIC", "-ffp-contract=fast", *fma, "-w",
             "-I", SHIM, "-I", src, "-include", os.path.join(SHIM, "kernel_env.h")]
    drv = os.path.join(OUT, "ref_driver.o")
    drv_src = os.path.join(HERE, "ref_driver.cpp")
    if force or not os.path.exists(drv) or os.path.getmtime(drv) < os.path.getmtime(drv_src):
        subprocess.run(["g++", *flags, "-c", drv_src, "-o", drv], check=True)
    built = []
    for name, d in MODELS.items():
        so = lib_path(name)
        if os.path.exists(so) and not force:
            built.append(so)
            continue
        obj = os.path.join(OUT, "kernels_%s.o" % name)
        sed = subprocess.Popen(["sed", "/^void run_mcmc/,$d", os.path.join(src, "gpu_mcmc.cu")],
                               stdout=subprocess.PIPE)
        cc = subprocess.run(["g++", "-x", "c++", *flags, "-I", os.path.join(REF_ROOT, d),
                             "-c", "-", "-o", obj], stdin=sed.stdout)
        sed.stdout.close()
        if sed.wait() != 0 or cc.returncode != 0:
            raise RuntimeError("compiling the reference kernels for %s failed" % name)
        subprocess.run(["g++", "-shared", "-o", so, obj, drv, "-lm"], check=True)
        built.append(so)
    return built


if __name__ == "__main__":
    if "--clean" in sys.argv and os.path.isdir(OUT):
        shutil.rmtree(OUT)
    print("\n".join(build(force="--force" in sys.argv)) or "reference tree not present")
