"""Python handle over the coupled-cluster driver of the C ABI (include/gbx_cc.h)."""
import ctypes

import numpy as np
import torch

from ._lib import lib, check

CCD, CCSD = 0, 1
FP64, SPLIT = 0, 1


class Config(ctypes.Structure):
    """gbx_cc_config."""
    _fields_ = [("nocc", ctypes.c_int), ("nvir", ctypes.c_int), ("nirrep", ctypes.c_int), ("max_block", ctypes.c_int),
                ("min_block", ctypes.c_int), ("method", ctypes.c_int), ("engine", ctypes.c_int),
                ("slices", ctypes.c_int), ("use_graph", ctypes.c_int), ("seed", ctypes.c_uint64),
                ("eps_occ_lo", ctypes.c_double), ("eps_occ_hi", ctypes.c_double), ("eps_vir_lo", ctypes.c_double),
                ("eps_vir_hi", ctypes.c_double), ("v_scale", ctypes.c_double), ("v_decay", ctypes.c_double)]


class Stats(ctypes.Structure):
    """gbx_cc_stats."""
    _fields_ = [("flops_per_iter", ctypes.c_double), ("gemm_flops_per_iter", ctypes.c_double),
                ("resident_bytes", ctypes.c_double), ("ncontractions", ctypes.c_int), ("nsums", ctypes.c_int),
                ("nblocks_occ", ctypes.c_int), ("nblocks_vir", ctypes.c_int), ("launches_per_iter", ctypes.c_int)]


def config(**kw):
    c = Config()
    lib().gbx_cc_default_config(ctypes.byref(c))
    for k, v in kw.items():
        if k == "method":
            v = {"ccd": CCD, "ccsd": CCSD}.get(v, v)
        if k == "engine":
            v = {"fp64": FP64, "split": SPLIT}.get(v, v)
        setattr(c, k, v)
    return c


def _stream(stream):
    s = stream if stream is not None else torch.cuda.current_stream()
    return ctypes.c_void_p(s.cuda_stream)


class Job:
    def __init__(self, stream=None, **kw):
        self.cfg = config(**kw)
        self.handle = ctypes.c_void_p()
        check(lib().gbx_cc_create(ctypes.byref(self.cfg), _stream(stream), ctypes.byref(self.handle)))

    @property
    def n(self):
        return self.cfg.nocc + self.cfg.nvir

    def iterate(self, niter, stream=None):
        e = np.zeros(niter)
        check(lib().gbx_cc_iterate(self.handle, niter, e.ctypes.data_as(ctypes.c_void_p), _stream(stream)))
        return e

    def enqueue(self, niter, stream=None):
        check(lib().gbx_cc_enqueue(self.handle, niter, _stream(stream)))

    def energies(self):
        cnt = ctypes.c_int(4096)
        e = np.zeros(4096)
        check(lib().gbx_cc_energies(self.handle, e.ctypes.data_as(ctypes.c_void_p), ctypes.byref(cnt)))
        return e[: cnt.value]

    def stats(self):
        s = Stats()
        check(lib().gbx_cc_stats_get(self.handle, ctypes.byref(s)))
        return s

    def orbitals(self):
        irr = np.zeros(self.n, dtype=np.int32)
        eps = np.zeros(self.n)
        check(lib().gbx_cc_get_orbitals(self.handle, irr.ctypes.data_as(ctypes.c_void_p),
                                        eps.ctypes.data_as(ctypes.c_void_p)))
        return irr, eps

    def amplitudes(self, stream=None):
        o, v = self.cfg.nocc, self.cfg.nvir
        t1 = np.zeros((o, v))
        t2 = np.zeros((o, o, v, v))
        check(lib().gbx_cc_get_amplitudes(self.handle, t1.ctypes.data_as(ctypes.c_void_p),
                                          t2.ctypes.data_as(ctypes.c_void_p), _stream(stream)))
        return t1, t2

    def close(self):
        if getattr(self, "handle", None) and self.handle.value:
            lib().gbx_cc_destroy(self.handle)
            self.handle = ctypes.c_void_p()

    def __del__(self):
        self.close()
