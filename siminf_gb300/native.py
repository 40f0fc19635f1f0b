"""Loads libsiminf_gb300.so and declares the C ABI of include/siminf_gb300.h.

There is no CPU fallback: if the library is missing, or no CUDA device is
visible, every entry point fails loudly.
"""
import ctypes as C
import os

import numpy as np

from . import abi

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libsiminf_gb300.so")

_lib = None


def lib():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(
            "libsiminf_gb300.so is not built (expected at %s); run "
            "`python -m siminf_gb300.build` or __graft_entry__.build()" % LIB_PATH)
    L = C.CDLL(LIB_PATH)
    vp = C.c_void_p
    L.siminf_gpu_model_builtin.argtypes = [C.c_char_p, C.POINTER(vp)]
    L.siminf_gpu_model_builtin.restype = C.c_int
    L.siminf_gpu_model_load.argtypes = [C.c_char_p, C.POINTER(vp)]
    L.siminf_gpu_model_load.restype = C.c_int
    L.siminf_gpu_model_dims.argtypes = [vp, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                        C.POINTER(C.c_int)]
    L.siminf_gpu_model_free.argtypes = [vp]
    L.siminf_gpu_model_free.restype = None
    for name in ("siminf_gpu_run_solver_ssm", "siminf_gpu_run_solver_mssm"):
        getattr(L, name).argtypes = [vp, vp]
        getattr(L, name).restype = C.c_int
    L.siminf_gpu_run_solver_ssm_noalloc.argtypes = [vp, vp, vp]
    L.siminf_gpu_run_solver_ssm_noalloc.restype = C.c_int
    L.siminf_gpu_run_batch.argtypes = [C.POINTER(abi.BatchJob), C.c_int, vp,
                                       C.POINTER(abi.BatchOptions)]
    L.siminf_gpu_run_batch.restype = C.c_int
    L.siminf_gpu_server_create.argtypes = [C.POINTER(abi.ServerOptions), C.POINTER(vp)]
    L.siminf_gpu_server_create.restype = C.c_int
    L.siminf_gpu_server_submit.argtypes = [vp, C.POINTER(abi.Request)]
    L.siminf_gpu_server_submit.restype = C.c_int
    L.siminf_gpu_server_wait.argtypes = [vp, C.POINTER(abi.Request), C.c_double]
    L.siminf_gpu_server_wait.restype = C.c_int
    L.siminf_gpu_server_load.argtypes = [vp, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                         C.POINTER(C.c_longlong)]
    L.siminf_gpu_server_load.restype = C.c_int
    L.siminf_gpu_server_free.argtypes = [vp]
    L.siminf_gpu_server_free.restype = None
    L.siminf_gpu_run_solver_ex.argtypes = [vp, vp, C.POINTER(abi.Options)]
    L.siminf_gpu_run_solver_ex.restype = C.c_int
    L.siminf_gpu_plan_create_ex.argtypes = [vp, vp, C.POINTER(abi.Options), C.POINTER(vp)]
    L.siminf_gpu_plan_create_ex.restype = C.c_int
    L.siminf_gpu_schedule.argtypes = [vp, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                      C.POINTER(C.c_longlong), C.POINTER(C.c_longlong),
                                      C.POINTER(C.c_int)]
    L.siminf_gpu_schedule.restype = C.c_int
    L.siminf_gpu_schedule_device.argtypes = [vp, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                             C.POINTER(C.c_longlong), C.POINTER(C.c_longlong),
                                             C.POINTER(C.c_int)]
    L.siminf_gpu_schedule_device.restype = C.c_int
    L.siminf_gpu_pmcmc_create.argtypes = [vp, vp, C.POINTER(abi.PfilterArgs),
                                          C.POINTER(abi.PmcmcArgs), C.POINTER(vp)]
    L.siminf_gpu_pmcmc_create.restype = C.c_int
    L.siminf_gpu_pmcmc_run.argtypes = [vp, C.c_int, vp]
    L.siminf_gpu_pmcmc_run.restype = C.c_int
    L.siminf_gpu_pmcmc_length.argtypes = [vp]
    L.siminf_gpu_pmcmc_length.restype = C.c_longlong
    L.siminf_gpu_pmcmc_free.argtypes = [vp]
    L.siminf_gpu_pmcmc_free.restype = None
    L.siminf_gpu_pfilter.argtypes = [vp, vp, C.POINTER(abi.PfilterArgs)]
    L.siminf_gpu_pfilter.restype = C.c_int
    L.siminf_gpu_individual_events_ex.argtypes = ([C.c_longlong] + [vp] * 6 +
                                                  [C.c_longlong, vp, vp])
    L.siminf_gpu_individual_events_ex.restype = C.c_int
    L.siminf_gpu_last_status.argtypes = [C.POINTER(abi.Status)]
    L.siminf_gpu_last_stats.argtypes = [C.POINTER(abi.Stats)]
    L.siminf_gpu_plan_create.argtypes = [vp, vp, C.POINTER(vp)]
    L.siminf_gpu_plan_create.restype = C.c_int
    L.siminf_gpu_plan_run.argtypes = [vp, vp]
    L.siminf_gpu_plan_run.restype = C.c_int
    L.siminf_gpu_plan_download.argtypes = [vp, vp]
    L.siminf_gpu_plan_download.restype = C.c_int
    L.siminf_gpu_plan_stats.argtypes = [vp, C.POINTER(abi.Stats)]
    L.siminf_gpu_plan_tune.argtypes = [vp, vp, C.c_int, C.POINTER(abi.TuneResult)]
    L.siminf_gpu_plan_tune.restype = C.c_int
    L.siminf_gpu_plan_free.argtypes = [vp]
    L.siminf_gpu_plan_free.restype = None
    L.siminf_gpu_release_cached.argtypes = []
    L.siminf_gpu_release_cached.restype = None
    pi = C.POINTER(C.c_int)
    L.siminf_gpu_trajectory_u.argtypes = [vp, C.c_int, C.c_int, C.c_int, pi, C.c_int, pi,
                                          C.c_int, pi, vp, C.POINTER(abi.ReduceStats)]
    L.siminf_gpu_trajectory_u.restype = C.c_int
    L.siminf_gpu_trajectory_v.argtypes = [vp, C.c_int, C.c_int, C.c_int, pi, C.c_int, pi,
                                          C.c_int, C.POINTER(C.c_double), vp,
                                          C.POINTER(abi.ReduceStats)]
    L.siminf_gpu_trajectory_v.restype = C.c_int
    L.siminf_gpu_prevalence.argtypes = [vp, C.c_int, C.c_int, C.c_int,
                                        C.POINTER(abi.PrevalenceSpec), pi, C.c_int,
                                        C.POINTER(C.c_double), vp, C.POINTER(abi.ReduceStats)]
    L.siminf_gpu_prevalence.restype = C.c_int
    L.siminf_gpu_plan_outputs.argtypes = [vp, C.POINTER(vp), C.POINTER(vp), pi]
    L.siminf_gpu_plan_outputs.restype = C.c_int
    L.siminf_gpu_sort_events.argtypes = [C.c_longlong, pi, pi, pi, pi, pi,
                                         C.POINTER(C.c_double), pi, pi, vp,
                                         C.POINTER(abi.ReduceStats)]
    L.siminf_gpu_sort_events.restype = C.c_int
    L.siminf_gpu_plan_day_max.argtypes = [vp, vp, C.POINTER(C.c_uint)]
    L.siminf_gpu_plan_day_max.restype = C.c_int
    L.siminf_gpu_individual_events.argtypes = [C.c_longlong, pi, pi, pi, pi, pi, pi, vp,
                                               C.POINTER(abi.ReduceStats)]
    L.siminf_gpu_individual_events.restype = C.c_int
    _lib = L
    return L


EXPORTS = (
    "siminf_gpu_model_builtin", "siminf_gpu_model_dims", "siminf_gpu_model_free",
    "siminf_gpu_run_solver_ssm", "siminf_gpu_run_solver_mssm", "siminf_gpu_run_solver_ex",
    "siminf_gpu_plan_create_ex", "siminf_gpu_last_status",
    "siminf_gpu_last_stats", "siminf_gpu_plan_create", "siminf_gpu_plan_run",
    "siminf_gpu_plan_download", "siminf_gpu_plan_stats", "siminf_gpu_plan_free",
    "siminf_gpu_plan_profile", "siminf_gpu_schedule", "siminf_gpu_schedule_device",
    "siminf_gpu_pfilter",
    "siminf_gpu_run_solver_ssm_noalloc", "siminf_gpu_run_batch",
    "siminf_gpu_server_create", "siminf_gpu_server_submit", "siminf_gpu_server_wait",
    "siminf_gpu_server_load", "siminf_gpu_server_free", "siminf_gpu_plan_tune",
    "siminf_gpu_release_cached", "siminf_gpu_trajectory_u", "siminf_gpu_trajectory_v",
    "siminf_gpu_prevalence", "siminf_gpu_plan_outputs", "siminf_gpu_sort_events",
    "siminf_gpu_plan_day_max", "siminf_gpu_individual_events",
    "siminf_gpu_individual_events_ex", "siminf_gpu_model_load",
    "siminf_gpu_pmcmc_create", "siminf_gpu_pmcmc_run", "siminf_gpu_pmcmc_length",
    "siminf_gpu_pmcmc_free",
)


def last_status():
    st = abi.Status()
    lib().siminf_gpu_last_status(C.byref(st))
    return st


def last_stats():
    st = abi.Stats()
    lib().siminf_gpu_last_stats(C.byref(st))
    return st


def check(code):
    if code != 0:
        st = last_status()
        raise abi.SimInfError(code, st.message.decode(errors="replace"))


def schedule(holder, device=False):
    """Wave planning of an args holder, on the host (siminf_gpu_schedule)
    or on the GPU (siminf_gpu_schedule_device): (days, waves, e1, e2,
    per-event wave array)."""
    import numpy as np
    n = max(1, holder.args.len)
    wave = np.zeros(n, dtype=np.int32)
    days, waves = C.c_int(), C.c_int()
    e1, e2 = C.c_longlong(), C.c_longlong()
    fn = lib().siminf_gpu_schedule_device if device else lib().siminf_gpu_schedule
    check(fn(C.cast(holder.ref(), C.c_void_p), C.byref(days), C.byref(waves), C.byref(e1),
             C.byref(e2), wave.ctypes.data_as(C.POINTER(C.c_int))))
    return days.value, waves.value, e1.value, e2.value, wave[:holder.args.len]


class DeviceModel:
    """A device model compiled into the library (siminf_gpu_model_builtin)."""

    def __init__(self, name):
        self.name = name
        h = C.c_void_p()
        check(lib().siminf_gpu_model_builtin(name.encode(), C.byref(h)))
        self.handle = h

    def dims(self):
        nc, nt, nd = C.c_int(), C.c_int(), C.c_int()
        lib().siminf_gpu_model_dims(self.handle, C.byref(nc), C.byref(nt), C.byref(nd))
        return nc.value, nt.value, nd.value

    def __del__(self):
        if getattr(self, "handle", None) and _lib is not None:
            _lib.siminf_gpu_model_free(self.handle)
            self.handle = None


_models = {}
_code_models = {}


def register_model_code(name, c_code, Nc, Nt, Nd, Ngd, pts_local=None):
    """Make `name` a device model compiled from model C code (devmodel),
    compiled and loaded the first time an entry point asks for it."""
    _code_models[name] = (c_code, Nc, Nt, Nd, Ngd, pts_local)


def load_device_model(name, path):
    """Load a device model library built by devmodel.compile
    (siminf_gpu_model_load) and register it under `name`."""
    dm = DeviceModel.__new__(DeviceModel)
    dm.name = name
    h = C.c_void_p()
    check(lib().siminf_gpu_model_load(os.fsencode(path), C.byref(h)))
    dm.handle = h
    _models[name] = dm
    return dm


def device_model(name):
    if name not in _models:
        if name in _code_models:
            from . import devmodel
            devmodel.load(name, *_code_models[name])
        else:
            _models[name] = DeviceModel(name)
    return _models[name]


class Plan:
    """A device-resident run (siminf_gpu_plan_*): inputs uploaded once,
    run() repeats the whole horizon on the GPU, download() fills the
    holder's U/V buffers."""

    def __init__(self, holder, model_name, cap_transfers=False, **options):
        """options: further siminf_gpu_options fields (heavy_rate,
        two_pass, gdata_per_replicate, max_node_day_transitions, streamed,
        ssa_variant, wave_block, heavy_lanes)."""
        self.holder = holder
        self.model = device_model(model_name)
        h = C.c_void_p()
        opt = abi.Options(cap_transfers=int(bool(cap_transfers)), **options)
        check(lib().siminf_gpu_plan_create_ex(C.cast(holder.ref(), C.c_void_p),
                                              self.model.handle, C.byref(opt), C.byref(h)))
        self.handle = h

    def run(self, stream=None):
        check(lib().siminf_gpu_plan_run(self.handle, stream))

    def download(self):
        check(lib().siminf_gpu_plan_download(self.handle, C.cast(self.holder.ref(), C.c_void_p)))

    def tune(self, probe_days=16, stream=None):
        """Autotune the launch layout (heavy threshold, one- or two-pass
        days, SSA register budget, lanes a warp for the heaviest nodes,
        wavefront block) on the first probe_days
        days (siminf_gpu_plan_tune; negative: a new search even if the size
        class has a cached choice); returns the TuneResult."""
        r = abi.TuneResult()
        check(lib().siminf_gpu_plan_tune(self.handle, stream, int(probe_days), C.byref(r)))
        return r

    def day_max(self, stream=None):
        """Per day, the most transitions any node fired (one recording run,
        siminf_gpu_plan_day_max)."""
        out = np.zeros(self.stats().days, dtype=np.uint32)
        check(lib().siminf_gpu_plan_day_max(self.handle, stream,
                                            out.ctypes.data_as(C.POINTER(C.c_uint))))
        return out

    def stats(self):
        st = abi.Stats()
        lib().siminf_gpu_plan_stats(self.handle, C.byref(st))
        return st

    def close(self):
        if getattr(self, "handle", None):
            lib().siminf_gpu_plan_free(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
