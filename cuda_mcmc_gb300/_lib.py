"""ctypes access to the model libraries (libcmc_<model>.so).

The libraries are built in-tree (cuda_mcmc_gb300/_lib/) by ``_build.build()``.
Loading never falls back to anything: a missing or unloadable library raises.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

from . import _build

_libs = {}
_lock = threading.Lock()

CMC_OK, CMC_ERR_ARG, CMC_ERR_CUDA, CMC_ERR_STREAM, CMC_ERR_MODEL, CMC_ERR_NOMEM, \
    CMC_ERR_UNSUPPORTED, CMC_ERR_TIMEOUT, CMC_ERR_CANCELLED = range(9)
CMC_RNG_CURAND, CMC_RNG_INJECTED = 0, 1
CMC_PROP_SINGLE, CMC_PROP_BLOCK = 0, 1
MODE_MODCHI2, MODE_MODEL = 1, 2


class McmcError(RuntimeError):
    """A C-ABI call returned a non-zero cmc_status."""

    def __init__(self, code, msg):
        super().__init__("cuda_mcmc error %d: %s" % (code, msg))
        self.code = code


_vp = C.c_void_p


class CmcJob(C.Structure):
    """Mirror of ``cmc_job`` (cuda_mcmc_gb300/csrc/cmc_job.h); pointers are
    device addresses."""
    _fields_ = [
        ("ncoor", C.c_int), ("ndat", C.c_int), ("nicoor", C.c_int), ("nidat", C.c_int),
        ("ndatm", C.c_int), ("nptot", C.c_int), ("nprm", C.c_int), ("nadj", C.c_int),
        ("npass", C.c_int), ("nbeta", C.c_int), ("nseq", C.c_int), ("imodel", C.c_int),
        ("do_init", C.c_int), ("nburn", C.c_int), ("niter", C.c_int), ("itr0", C.c_int),
        ("niter_total", C.c_int), ("rng_mode", C.c_int), ("seed", C.c_ulonglong),
        ("coor", _vp), ("dat", _vp), ("std2r", _vp), ("icoor", _vp), ("idat", _vp),
        ("pdescr", _vp), ("ivar", _vp), ("invar", _vp), ("pmint", _vp), ("pmaxt", _vp),
        ("beta", _vp), ("hidat", C.c_int * 4),
        ("pcur", _vp), ("chi2c", _vp), ("flag", _vp), ("ptent", _vp), ("ptentn", _vp),
        ("pstp", _vp), ("n_acpt", _vp), ("n_exch", _vp), ("n_cnt", _vp), ("n_hist", _vp),
        ("tcur", _vp), ("rndst", _vp),
        ("pout", _vp), ("tout", _vp), ("chi2", _vp), ("datm", _vp), ("chi2m", _vp),
        ("inj_u", _vp), ("inj_n", _vp), ("inj_lu", C.c_int), ("inj_ln", C.c_int),
        ("inj_cur", _vp),
        ("work", _vp), ("work_bytes", C.c_size_t),
        ("status", _vp),
        ("prop_mode", C.c_int), ("prop_reserved", C.c_int), ("prop_chol", _vp),
        ("seq_offset", C.c_int), ("nseq_total", C.c_int),
    ]


_fp = C.POINTER(C.c_float)
_ip = C.POINTER(C.c_int)
_u8p = C.POINTER(C.c_ubyte)

# argument types of the reference's entry points (src/mcmc.h:7-32)
MCMC_CUDA_ARGS = ([_fp, _fp, _fp, _ip, _ip, _fp, _fp, _ip, _ip, _ip, _fp, _fp, _fp, _fp, _ip, _fp,
                   _fp, _ip, _ip, _ip, _ip, _ip, _ip, _fp, _fp, _fp, _ip, _fp, _u8p,
                   C.c_ulonglong] + [C.c_int] * 14)
CALC_MODCHI2_ARGS = [_fp, _fp, _fp, _ip, _ip, _fp, _fp, _fp, _fp, _ip] + [C.c_int] * 9
CALC_MODEL_ARGS = [_fp, _ip, _fp, _fp] + [C.c_int] * 8

EXPORTS = ("mcmc_cuda", "mcmc_cuda_v2", "calc_modchi2", "calc_modchi2_v2", "calc_model",
           "calc_model_v2", "cmc_last_error", "cmc_model_name", "cmc_abi_version",
           "cmc_sizeof_job", "cmc_reset_gpu", "cmc_work_bytes", "cmc_run", "cmc_eval",
           "cmc_query_config", "cmc_set_config", "cmc_set_layout", "cmc_set_spread",
           "cmc_query_spread", "cmc_batch_work_bytes",
           "cmc_batch_prepare",
           "cmc_batch_run", "cmc_batch_info", "cmc_batch_free", "cmc_batch_run_class",
           "cmc_batch_cancel",
           "cmc_batch_set_class")


def _declare(L):
    L.mcmc_cuda.argtypes = MCMC_CUDA_ARGS
    L.mcmc_cuda.restype = None
    L.mcmc_cuda_v2.argtypes = MCMC_CUDA_ARGS
    L.mcmc_cuda_v2.restype = C.c_int
    L.calc_modchi2.argtypes = CALC_MODCHI2_ARGS
    L.calc_modchi2.restype = None
    L.calc_modchi2_v2.argtypes = CALC_MODCHI2_ARGS
    L.calc_modchi2_v2.restype = C.c_int
    L.calc_model.argtypes = CALC_MODEL_ARGS
    L.calc_model.restype = None
    L.calc_model_v2.argtypes = CALC_MODEL_ARGS
    L.calc_model_v2.restype = C.c_int
    L.cmc_last_error.restype = C.c_char_p
    L.cmc_model_name.restype = C.c_char_p
    L.cmc_abi_version.restype = C.c_int
    L.cmc_sizeof_job.restype = C.c_int
    L.cmc_reset_gpu.restype = C.c_int
    L.cmc_work_bytes.argtypes = [C.POINTER(CmcJob), C.c_int]
    L.cmc_work_bytes.restype = C.c_size_t
    L.cmc_run.argtypes = [C.POINTER(CmcJob), C.c_void_p]
    L.cmc_run.restype = C.c_int
    L.cmc_eval.argtypes = [C.POINTER(CmcJob), C.c_int, C.c_void_p]
    L.cmc_eval.restype = C.c_int
    L.cmc_query_config.argtypes = [C.POINTER(CmcJob), _ip, _ip, _ip, _ip,
                                   C.POINTER(C.c_size_t), _ip]
    L.cmc_query_config.restype = C.c_int
    L.cmc_set_config.argtypes = [C.c_int, C.c_int, C.c_int]
    L.cmc_set_config.restype = None
    L.cmc_set_layout.argtypes = [C.c_int]
    L.cmc_set_layout.restype = None
    L.cmc_set_spread.argtypes = [C.c_int, C.c_int]
    L.cmc_set_spread.restype = None
    L.cmc_query_spread.argtypes = [C.POINTER(CmcJob), _ip, _ip]
    L.cmc_query_spread.restype = C.c_int
    L.cmc_batch_work_bytes.argtypes = [C.POINTER(CmcJob), C.c_int]
    L.cmc_batch_work_bytes.restype = C.c_size_t
    L.cmc_batch_prepare.argtypes = [C.POINTER(CmcJob), C.c_int, C.c_void_p, C.c_size_t,
                                    C.c_void_p]
    L.cmc_batch_prepare.restype = C.c_void_p
    L.cmc_batch_run.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p]
    L.cmc_batch_run.restype = C.c_int
    L.cmc_batch_info.argtypes = [C.c_void_p, C.c_int, _ip, _ip, _ip, _ip, _ip, _ip,
                                 C.POINTER(C.c_size_t)]
    L.cmc_batch_info.restype = C.c_int
    L.cmc_batch_free.argtypes = [C.c_void_p]
    L.cmc_batch_free.restype = None
    L.cmc_batch_cancel.argtypes = [C.c_void_p]
    L.cmc_batch_cancel.restype = C.c_int
    L.cmc_batch_run_class.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                      C.c_void_p]
    L.cmc_batch_run_class.restype = C.c_int
    L.cmc_batch_set_class.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int,
                                      C.c_void_p]
    L.cmc_batch_set_class.restype = C.c_int
    if hasattr(L, "cmc_grad"):          # Sgr A* library only
        L.cmc_grad_work_bytes.argtypes = [C.POINTER(CmcJob)]
        L.cmc_grad_work_bytes.restype = C.c_size_t
        L.cmc_grad.argtypes = [C.POINTER(CmcJob), C.c_void_p, C.c_void_p]
        L.cmc_grad.restype = C.c_int
        L.cmc_fisher_work_bytes.argtypes = [C.POINTER(CmcJob)]
        L.cmc_fisher_work_bytes.restype = C.c_size_t
        L.cmc_fisher.argtypes = [C.POINTER(CmcJob), C.c_void_p, C.c_void_p]
        L.cmc_fisher.restype = C.c_int
    if hasattr(L, "cmc_module_set"):    # module library only
        L.cmc_module_set.argtypes = [C.c_char_p]
        L.cmc_module_set.restype = C.c_int
    if L.cmc_sizeof_job() != C.sizeof(CmcJob):
        raise RuntimeError("cmc_job layout mismatch between %s and _lib.CmcJob" % L._name)


def load_path(path: str, name: str = None):
    """Load a model library by path (e.g. a user plugin built by build_plugin)."""
    key = os.path.abspath(path)
    with _lock:
        if key not in _libs:
            if not os.path.exists(key):
                raise FileNotFoundError(
                    "cuda_mcmc_gb300: model library %s is missing; run "
                    "cuda_mcmc_gb300._build.build() (there is no CPU fallback)" % key)
            L = C.CDLL(key)
            _declare(L)
            _libs[key] = L
        return _libs[key]


def load(model: str = "sgra", build: bool = True):
    """Load the built-in library of ``model`` (sgra, rosenbrock, solvsys, nlsys),
    building it first when ``build`` is true and it is out of date."""
    path = _build.lib_path(model)
    if build and (model in ("sgra", "module") or model in _build.BUILTIN_PLUGINS):
        if not os.path.exists(path) or not os.path.exists(path + ".stamp"):
            _build.build([model])
    return load_path(path, model)


def load_module(module_file: str, tag: str = None):
    """A model library whose kernels come from ``module_file`` (a cubin or
    PTX built by _build.build_module from a model.cuh): a private copy of
    libcmc_module.so is loaded (each copy holds one module), pointed at the
    file and returned."""
    import shutil
    import tempfile
    src = _build.lib_path("module")
    if not os.path.exists(src) or not os.path.exists(src + ".stamp"):
        _build.build(["module"])
    tag = tag or os.path.splitext(os.path.basename(module_file))[0]
    d = os.path.join(tempfile.gettempdir(), "cmc_module_%d" % os.getpid())
    os.makedirs(d, exist_ok=True)
    dst = os.path.join(d, "libcmc_module_%s.so" % tag)
    if not os.path.exists(dst):
        shutil.copyfile(src, dst)
    L = load_path(dst, tag)
    check(L, L.cmc_module_set(os.path.abspath(module_file).encode()))
    return L


def check(L, rc):
    if rc != CMC_OK:
        raise McmcError(rc, L.cmc_last_error().decode(errors="replace"))
    return rc


def loaded_paths():
    return sorted(_libs)
