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

For the same models it also builds the reference's GPU code, unchanged:
src/gpu_mcmc.cu (all of it, with the example's model.cuh) for sm_103a as
``oracle/_ref/ref_gpu_<name>.cubin`` and as PTX (``.ptx``, loaded by the
driver's JIT where the cubin is absent), plus ``ref_gpu_layout.json``, the
byte offsets of the reference's CMcmcFit members printed by
oracle/ref_layout.cu.  oracle/ref_gpu.py loads those kernels through the CUDA
driver API and launches them in run_mcmc's order: the reference's own CUDA
build, run on the GPU beside this library.

The reference tree is found through the environment variable
CUDA_MCMC_REFERENCE; a build made with it records the path in
``oracle/_ref/source_root`` so that later rebuilds in the same checkout find
it again.  Without either, nothing is built.  Only the build container has
the reference tree: the CPU outputs generate the committed golden fixtures
(tests/golden/make_golden.py), and the GPU outputs (device code and a JSON
file, no host binaries) travel with the working tree to the GPU host.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
SHIM = os.path.join(HERE, "ref_shim")
_ROOT_FILE = os.path.join(OUT, "source_root")


def _ref_root():
    root = os.environ.get("CUDA_MCMC_REFERENCE", "")
    if not root and os.path.isfile(_ROOT_FILE):
        with open(_ROOT_FILE) as f:
            root = f.read().strip()
    return root


REF_ROOT = _ref_root()

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
    return bool(REF_ROOT) and os.path.isfile(os.path.join(REF_ROOT, "src", "gpu_mcmc.cu"))


def _remember_root():
    os.makedirs(OUT, exist_ok=True)
    with open(_ROOT_FILE, "w") as f:
        f.write(REF_ROOT + "\n")


def lib_path(name: str) -> str:
    return os.path.join(OUT, "libref_%s.so" % name)


def build(force: bool = False) -> list:
    if not available():
        return []
    _remember_root()
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


# ---- the reference's GPU build --------------------------------------------------

def gpu_paths(name: str) -> dict:
    return {"cubin": os.path.join(OUT, "ref_gpu_%s.cubin" % name),
            "ptx": os.path.join(OUT, "ref_gpu_%s.ptx" % name),
            "layout": os.path.join(OUT, "ref_gpu_layout.json")}


def _nvcc() -> str:
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    p = os.path.join(cuda, "bin", "nvcc")
    return p if os.path.exists(p) else "nvcc"


def build_gpu(force: bool = False) -> list:
    """src/gpu_mcmc.cu + examples/<m>/model.cuh for sm_103a (cubin and PTX),
    compiled as the reference's src/Makefile compiles it (nvcc defaults for
    device code: -O3, fused multiply-adds), and the CMcmcFit layout."""
    if not available():
        return []
    _remember_root()
    src = os.path.join(REF_ROOT, "src")
    out = []
    lay = gpu_paths("sgra")["layout"]
    if force or not os.path.exists(lay):
        exe = os.path.join(OUT, "ref_layout")
        subprocess.run([_nvcc(), "-std=c++17", "-w", "-I", src, "-o", exe,
                        os.path.join(HERE, "ref_layout.cu")], check=True)
        txt = subprocess.run([exe], check=True, capture_output=True, text=True).stdout
        os.remove(exe)
        with open(lay, "w") as f:
            f.write(txt)
    out.append(lay)
    for name, d in MODELS.items():
        p = gpu_paths(name)
        inc = ["-I", src, "-I", os.path.join(REF_ROOT, d)]
        for kind, flags in (("cubin", ["-cubin", "-arch=sm_103a"]),
                            ("ptx", ["-ptx", "-arch=compute_103a"])):
            if force or not os.path.exists(p[kind]):
                subprocess.run([_nvcc(), *flags, "-w", *inc, "-o", p[kind],
                                os.path.join(src, "gpu_mcmc.cu")], check=True)
            out.append(p[kind])
    return out


# ---- the reference's model.cuh files as modules of this library ------------------

PLUGIN_DIRS = {"sgra": "examples/sgra_model_fit", "rosenbrock": "examples/search_Rosenbrock",
               "solvsys": "examples/solvsys", "template": "template"}


def module_path(name: str) -> str:
    return os.path.join(OUT, "plugin_%s.cubin" % name)


def build_modules(force: bool = False) -> list:
    """The reference's four shipped model.cuh files, unchanged, each compiled
    with this library's module_plugin.cu (the sweep, batch and evaluation
    kernels of the plugin path) into oracle/_ref/plugin_<name>.cubin, which
    libcmc_module.so loads on the GPU host."""
    if not available():
        return []
    _remember_root()
    import importlib
    sys.path.insert(0, os.path.dirname(HERE))
    _build = importlib.import_module("cuda_mcmc_gb300._build")
    out = []
    for name, d in PLUGIN_DIRS.items():
        p = module_path(name)
        if force or not os.path.exists(p):
            # the Sgr A* file is heavy (Bessel functions in every model call):
            # kernels for 1 and 2 replicas per CTA keep its compile to minutes
            _build.build_module(os.path.join(REF_ROOT, d, "model.cuh"), p,
                                max_r=2 if name == "sgra" else 32)
        out.append(p)
    return out


# ---- the reference's Cython bridge -------------------------------------------------

def cython_path() -> str:
    return os.path.join(OUT, "mcmc_interf_ref.c")


def build_cython(force: bool = False) -> list:
    """src/mcmc_interf.pyx, unchanged, through Cython into C (without the
    .pyx source lines as comments).  The C compiles wherever numpy's headers
    and a "mcmc.h" are on the include path; the tests compile it against this
    repository's include/mcmc.h and link it with libcmc_sgra.so, the drop-in
    use of the bridge."""
    if not available():
        return []
    try:
        from Cython.Build import cythonize  # noqa: F401
    except ImportError:
        return []
    _remember_root()
    out = cython_path()
    if force or not os.path.exists(out):
        import tempfile
        tmp = tempfile.mkdtemp()
        pyx = os.path.join(tmp, "mcmc_interf.pyx")
        shutil.copyfile(os.path.join(REF_ROOT, "src", "mcmc_interf.pyx"), pyx)
        subprocess.run([sys.executable, "-m", "cython", "-3", "-X", "emit_code_comments=False",
                        "-X", "language_level=2", pyx, "-o", out], check=True,
                       capture_output=True)
        shutil.rmtree(tmp)
    return [out]


if __name__ == "__main__":
    if "--clean" in sys.argv and os.path.isdir(OUT):
        shutil.rmtree(OUT)
    force = "--force" in sys.argv
    print("\n".join(build(force=force) + build_gpu(force=force) + build_cython(force=force)
                    + build_modules(force=force))
          or "reference tree not found (set CUDA_MCMC_REFERENCE)")
