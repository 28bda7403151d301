"""Build the model libraries in-tree with nvcc for sm_103a.

Each model library ``cuda_mcmc_gb300/_lib/libcmc_<name>.so`` is linked from
one C-ABI object (lib_sgra.cu or lib_plugin.cu) plus one kernel-instance
object per replicas-per-CTA count R (inst_*.cu with -DCMC_R=R); all objects
of all libraries compile in parallel.

Built-in libraries: ``sgra`` (the fast Sgr A* path), the model.cuh plugins
shipped in cuda_mcmc_gb300/models/ (rosenbrock, solvsys, nlsys) and
``module``, the plugin C-ABI whose kernels come from a CUDA module file
loaded at run time (a model.cuh compiled elsewhere with
:func:`build_module`).  Any other plugin -- e.g. a reference example's
model.cuh -- is built with :func:`build_plugin`.
"""
from __future__ import annotations

import hashlib
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(os.path.dirname(PKG), "include")
MODELS_DIR = os.path.join(PKG, "models")
# CMC_LIB_DIR / CMC_NVCC_FLAGS let experiments build variants side by side
LIB_DIR = os.environ.get("CMC_LIB_DIR", os.path.join(PKG, "_lib"))
OBJ_DIR = os.path.join(LIB_DIR, "obj")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# replicas-per-CTA instances per library (must match each model's kMaxR)
R_VALUES = {"sgra": (1, 2, 3, 4, 5, 6, 7, 8)}
R_VALUES_PLUGIN = (1, 2, 4, 8, 16, 32)
BUILTIN_PLUGINS = ("rosenbrock", "solvsys", "nlsys")


def nvcc() -> str:
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    p = os.path.join(cuda, "bin", "nvcc")
    return p if os.path.exists(p) else "nvcc"


def _flags():
    return [*ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
            "-I", CSRC, "-I", INCLUDE, "--expt-relaxed-constexpr",
            *os.environ.get("CMC_NVCC_FLAGS", "").split()]


def _sources_digest(extra=()):
    h = hashlib.sha1(os.environ.get("CMC_NVCC_FLAGS", "").encode())
    for d in (CSRC, INCLUDE):
        for name in sorted(os.listdir(d)):
            if not os.path.isfile(os.path.join(d, name)):
                continue
            with open(os.path.join(d, name), "rb") as f:
                h.update(name.encode())
                h.update(f.read())
    for p in extra:
        with open(p, "rb") as f:
            h.update(f.read())
    return h.hexdigest()[:16]


def lib_path(name: str) -> str:
    return os.path.join(LIB_DIR, "libcmc_%s.so" % name)


def _jobs_for(name, plugin_file=None):
    """(object path, nvcc args) for every object of one library."""
    jobs = []
    defs = []
    if name == "module":
        defs = ['-DCMC_PLUGIN_NAME="module"']
        for src, tag in (("lib_plugin.cu", "abi"), ("inst_module.cu", "launch")):
            o = os.path.join(OBJ_DIR, "module_%s.o" % tag)
            jobs.append((o, [nvcc(), *_flags(), *defs, "-c", os.path.join(CSRC, src), "-o", o]))
        return jobs
    if plugin_file is not None:
        defs = ['-DCMC_PLUGIN_FILE="%s"' % os.path.abspath(plugin_file),
                '-DCMC_PLUGIN_NAME="%s"' % name]
        abi_src, inst_src = os.path.join(CSRC, "lib_plugin.cu"), os.path.join(CSRC, "inst_plugin.cu")
    else:
        abi_src, inst_src = os.path.join(CSRC, "lib_%s.cu" % name), os.path.join(CSRC, "inst_%s.cu" % name)
    o = os.path.join(OBJ_DIR, "%s_abi.o" % name)
    jobs.append((o, [nvcc(), *_flags(), *defs, "-c", abi_src, "-o", o]))
    for r in (R_VALUES_PLUGIN if plugin_file is not None else R_VALUES[name]):
        o = os.path.join(OBJ_DIR, "%s_r%d.o" % (name, r))
        jobs.append((o, [nvcc(), *_flags(), *defs, "-DCMC_R=%d" % r, "-c", inst_src, "-o", o]))
    return jobs


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed:\n%s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return r.stdout + r.stderr


def build(names=None, force: bool = False, jobs: int = 0, verbose: bool = False) -> dict:
    """Build the built-in libraries (all by default); returns {name: path}."""
    names = list(names) if names else ["sgra", *BUILTIN_PLUGINS, "module"]
    os.makedirs(OBJ_DIR, exist_ok=True)
    plan = {}
    for n in names:
        plugin = None if n in ("sgra", "module") else os.path.join(MODELS_DIR, "%s.cuh" % n)
        plan[n] = (plugin, _jobs_for(n, plugin))
    return _build_plan(plan, force, jobs, verbose)


def build_module(model_cuh: str, out: str, ptx: bool = False, max_r: int = 32) -> str:
    """Compile a model.cuh (reference plugin convention, unchanged) with
    module_plugin.cu into a CUDA module file (cubin, or PTX with ``ptx``)
    that libcmc_module.so loads at run time (cmc_module_set), with kernels
    for 1 .. max_r replicas per CTA."""
    if not os.path.isfile(model_cuh):
        raise FileNotFoundError(model_cuh)
    kind = ["-ptx", "-arch=compute_103a"] if ptx else ["-cubin", "-arch=sm_103a"]
    os.makedirs(os.path.dirname(os.path.abspath(out)), exist_ok=True)
    tmp = out + ".tmp%d" % os.getpid()
    _run([nvcc(), *kind, "-O3", "-std=c++17", "-I", CSRC, "-I", INCLUDE,
          "--expt-relaxed-constexpr", "-w",
          '-DCMC_PLUGIN_FILE="%s"' % os.path.abspath(model_cuh), "-DCMC_MODULE_MAX_R=%d" % max_r,
          os.path.join(CSRC, "module_plugin.cu"), "-o", tmp])
    os.replace(tmp, out)
    return out


def build_plugin(model_cuh: str, name: str, force: bool = False, jobs: int = 0) -> str:
    """Compile a user's model.cuh (reference plugin convention, unchanged)
    into libcmc_<name>.so and return its path."""
    if not os.path.isfile(model_cuh):
        raise FileNotFoundError(model_cuh)
    os.makedirs(OBJ_DIR, exist_ok=True)
    return _build_plan({name: (model_cuh, _jobs_for(name, model_cuh))}, force, jobs, False)[name]


def _build_plan(plan, force, jobs, verbose):
    out = {}
    todo = []
    stamps = {}
    for name, (plugin, objs) in plan.items():
        digest = _sources_digest([plugin] if plugin else [])
        stamp = lib_path(name) + ".stamp"
        stamps[name] = (stamp, digest)
        if (not force and os.path.exists(lib_path(name)) and os.path.exists(stamp)
                and open(stamp).read().strip() == digest):
            out[name] = lib_path(name)
            continue
        todo.append(name)
    if todo:
        cmds = [cmd for n in todo for (_, cmd) in plan[n][1]]
        workers = jobs or max(1, min(len(cmds), os.cpu_count() or 4))
        with ThreadPoolExecutor(workers) as ex:
            logs = list(ex.map(_run, cmds))
        if verbose:
            for l in logs:
                if l.strip():
                    print(l)
        for n in todo:
            objs = [o for (o, _) in plan[n][1]]
            tmp = lib_path(n) + ".tmp%d" % os.getpid()
            _run([nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"])
            os.replace(tmp, lib_path(n))
            with open(stamps[n][0], "w") as f:
                f.write(stamps[n][1])
            out[n] = lib_path(n)
    return out


def clean():
    if os.path.isdir(LIB_DIR):
        shutil.rmtree(LIB_DIR)


if __name__ == "__main__":
    import time
    t = time.time()
    res = build(sys.argv[1:] or None, force="--force" in os.environ.get("CMC_BUILD_FLAGS", ""),
                verbose=True)
    print(res, "%.1fs" % (time.time() - t))
