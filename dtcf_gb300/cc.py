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
                ("slices", ctypes.c_int), ("use_graph", ctypes.c_int), ("split_all", ctypes.c_int),
                ("seed", ctypes.c_uint64),
                ("eps_occ_lo", ctypes.c_double), ("eps_occ_hi", ctypes.c_double), ("eps_vir_lo", ctypes.c_double),
                ("eps_vir_hi", ctypes.c_double), ("v_scale", ctypes.c_double), ("v_decay", ctypes.c_double),
                ("autotune", ctypes.c_int)]


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

    def gemm_shapes(self):
        cnt = ctypes.c_int(0)
        check(lib().gbx_cc_gemm_shapes(self.handle, None, ctypes.byref(cnt)))
        out = np.zeros((cnt.value, 3), dtype=np.int64)
        check(lib().gbx_cc_gemm_shapes(self.handle, out.ctypes.data_as(ctypes.c_void_p), ctypes.byref(cnt)))
        return out

    def amplitude_elems(self):
        n1, n2 = ctypes.c_int64(), ctypes.c_int64()
        check(lib().gbx_cc_amplitude_elems(self.handle, ctypes.byref(n1), ctypes.byref(n2)))
        return n1.value, n2.value

    def set_amplitudes(self, t1_ptr, t2_ptr, stream=None):
        """Host pointers (ints) of tile-storage amplitudes; copies are enqueued."""
        check(lib().gbx_cc_set_amplitudes(self.handle, ctypes.c_void_p(t1_ptr), ctypes.c_void_p(t2_ptr),
                                          _stream(stream)))

    def read_energy(self, host_ptr, stream=None):
        check(lib().gbx_cc_read_energy(self.handle, ctypes.c_void_p(host_ptr), _stream(stream)))

    def profile(self, stream=None):
        """One iteration step by step: list of dicts (name, kind, ms, flops, bytes)."""
        cap, nl = 512, 96
        ms = np.zeros(cap, dtype=np.float32)
        fl, by = np.zeros(cap), np.zeros(cap)
        kind = np.zeros(cap, dtype=np.int32)
        plan = np.zeros(cap, dtype=np.int32)
        names = ctypes.create_string_buffer(cap * nl)
        cnt = ctypes.c_int()
        P = lambda a: a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731
        check(lib().gbx_cc_profile(self.handle, cap, P(ms), P(fl), P(by), P(kind), P(plan), names, nl,
                                   ctypes.byref(cnt), _stream(stream)))
        out = []
        for i in range(min(cnt.value, cap)):
            nm = names.raw[i * nl:(i + 1) * nl].split(b"\0", 1)[0].decode()
            out.append(dict(name=nm, kind=int(kind[i]), ms=float(ms[i]), flops=float(fl[i]), bytes=float(by[i]),
                            plan=int(plan[i])))
        return out

    def plan_info(self, contraction):
        """dict(split_width, n_split, n_f64, slices) of one contraction's GEMMs."""
        v = [ctypes.c_int() for _ in range(4)]
        check(lib().gbx_cc_plan_info(self.handle, contraction, *[ctypes.byref(x) for x in v]))
        return dict(zip(("split_width", "n_split", "n_f64", "slices"), (x.value for x in v)))

    def time_gemm(self, contraction, reps=5, stream=None):
        """GEMM launches of one contraction alone: dict(ms, fp64_flops, tensor_flops, engine)."""
        ms = ctypes.c_float()
        f64, ten = ctypes.c_double(), ctypes.c_double()
        eng = ctypes.c_int()
        check(lib().gbx_cc_time_gemm(self.handle, contraction, reps, ctypes.byref(ms), ctypes.byref(f64),
                                     ctypes.byref(ten), ctypes.byref(eng), _stream(stream)))
        return dict(ms=ms.value, fp64_flops=f64.value, tensor_flops=ten.value, engine=eng.value)

    def contraction_error(self, contraction, stream=None):
        """(relative Frobenius error, max abs error) of one contraction of
        this job against a plain FP64 plan of it, on the current operands."""
        rel, mx = ctypes.c_double(), ctypes.c_double()
        check(lib().gbx_cc_contraction_error(self.handle, contraction, ctypes.byref(rel), ctypes.byref(mx),
                                             _stream(stream)))
        return rel.value, mx.value

    def program_info(self):
        """dict(records, levels, launches) of the persistent program (use_graph=2; zeros otherwise)."""
        v = [ctypes.c_int() for _ in range(3)]
        check(lib().gbx_cc_program_info(self.handle, *[ctypes.byref(x) for x in v]))
        return dict(zip(("records", "levels", "launches"), (x.value for x in v)))

    def close(self):
        if getattr(self, "handle", None) and self.handle.value:
            lib().gbx_cc_destroy(self.handle)
            self.handle = ctypes.c_void_p()

    def __del__(self):
        self.close()


def program_selftest(limit_cycles, stream=None):
    """Status of gbx_cc_program_selftest (GBX_ETIMEOUT when the bounded wait ran out, as it must)."""
    return lib().gbx_cc_program_selftest(limit_cycles, _stream(stream))
