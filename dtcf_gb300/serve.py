"""Serving loop for CC iteration requests (include/gbx_serve.h) over ctypes."""
import ctypes

from ._lib import lib, check
from .cc import Config


class ServeConfig(ctypes.Structure):
    """gbx_serve_config."""
    _fields_ = [("budget_bytes", ctypes.c_double), ("slots", ctypes.c_int), ("reserved", ctypes.c_int)]


class ServeResult(ctypes.Structure):
    """gbx_serve_result."""
    _fields_ = [("job", ctypes.c_int), ("iteration", ctypes.c_int), ("status", ctypes.c_int), ("slot", ctypes.c_int),
                ("arrival", ctypes.c_double), ("start", ctypes.c_double), ("end", ctypes.c_double),
                ("energy", ctypes.c_double)]


class ServeStats(ctypes.Structure):
    """gbx_serve_stats."""
    _fields_ = [("requests", ctypes.c_int), ("completed", ctypes.c_int), ("rejected", ctypes.c_int),
                ("timed_out", ctypes.c_int), ("jobs", ctypes.c_int), ("jobs_admitted", ctypes.c_int),
                ("jobs_rejected", ctypes.c_int), ("makespan_s", ctypes.c_double), ("iter_per_s", ctypes.c_double),
                ("latency_p50_s", ctypes.c_double), ("latency_p99_s", ctypes.c_double),
                ("latency_max_s", ctypes.c_double), ("service_p50_s", ctypes.c_double),
                ("peak_planned_bytes", ctypes.c_double), ("peak_measured_bytes", ctypes.c_double),
                ("build_s_total", ctypes.c_double), ("evictions", ctypes.c_int), ("restores", ctypes.c_int),
                ("evict_s_total", ctypes.c_double)]


class Server:
    """One serving run: add jobs, submit their iteration requests, run, read results."""

    def __init__(self, budget_bytes=160e9, slots=4):
        cfg = ServeConfig(budget_bytes, slots, 0)
        h = ctypes.c_void_p()
        check(lib().gbx_server_create(ctypes.byref(cfg), ctypes.byref(h)))
        self._h = h
        self.footprints = []

    def add_job(self, cfg):
        """cfg: a dtcf_gb300.cc.Config.  Returns the job id."""
        assert isinstance(cfg, Config)
        jid = ctypes.c_int()
        fp = ctypes.c_double()
        check(lib().gbx_server_add_job(self._h, ctypes.byref(cfg), ctypes.byref(jid), ctypes.byref(fp)))
        self.footprints.append(fp.value)
        return jid.value

    def submit(self, job, arrival_s):
        check(lib().gbx_server_submit(self._h, job, float(arrival_s)))

    def run(self, time_limit_s=0.0):
        check(lib().gbx_server_run(self._h, float(time_limit_s)))

    def results(self):
        n = ctypes.c_int(0)
        check(lib().gbx_server_results(self._h, None, ctypes.byref(n)))
        arr = (ServeResult * max(n.value, 1))()
        check(lib().gbx_server_results(self._h, ctypes.cast(arr, ctypes.c_void_p), ctypes.byref(n)))
        return [{f: getattr(arr[i], f) for f, _ in ServeResult._fields_} for i in range(n.value)]

    def stats(self):
        st = ServeStats()
        check(lib().gbx_server_stats(self._h, ctypes.byref(st)))
        return {f: getattr(st, f) for f, _ in ServeStats._fields_}

    def close(self):
        if getattr(self, "_h", None):
            lib().gbx_server_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()
