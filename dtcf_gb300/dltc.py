"""Python handle over the DLTC executor of the C ABI (include/gbx_dltc.h):
task_mul / task_sum over dense GA-layout tensors on the device, and the
residual tables (CCD-T2, CCSD-T1, CCSD-T2) as programs."""
import ctypes

import numpy as np
import torch

from ._lib import lib, check

MUL, SUM = 0, 1
CCD_T2, CCSD_T1, CCSD_T2 = 0, 1, 2
TABLES = {"ccd_t2": CCD_T2, "ccsd_t1": CCSD_T1, "ccsd_t2": CCSD_T2}
MAX_NAMES = 24
MODES = {"fp64": 0, "split": 1}
# IndexName values of the reference's normal build (DLTC/param.h): h1..h12, p1..p12
NAMES = ["h%d" % i for i in range(1, 13)] + ["p%d" % i for i in range(1, 13)]


class Dims(ctypes.Structure):
    """gbx_dltc_dims."""
    _fields_ = [("O", ctypes.c_int), ("V", ctypes.c_int), ("wbO", ctypes.c_int), ("wbV", ctypes.c_int),
                ("nocc_names", ctypes.c_int)]


class Expr(ctypes.Structure):
    """gbx_dltc_expr."""
    _fields_ = [("kind", ctypes.c_int), ("index", ctypes.c_int), ("layer", ctypes.c_int), ("c", ctypes.c_int),
                ("a", ctypes.c_int), ("b", ctypes.c_int), ("rc", ctypes.c_int), ("ra", ctypes.c_int),
                ("rb", ctypes.c_int), ("idc", ctypes.c_int * 4), ("ida", ctypes.c_int * 4), ("idb", ctypes.c_int * 4),
                ("coef", ctypes.c_double)]


def _iarr(x):
    a = np.ascontiguousarray(x, dtype=np.int32)
    return a, a.ctypes.data_as(ctypes.c_void_p)


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


def _stream(stream):
    s = stream if stream is not None else torch.cuda.current_stream()
    return ctypes.c_void_p(s.cuda_stream)


def dims(O, V, wbO, wbV, nocc_names=12):
    return Dims(O, V, wbO, wbV, nocc_names)


def mul_orders(idA, idB):
    """(m, n, k) name lists of a Multiplication (DLTC/expr.cc:13-67)."""
    a, ap = _iarr(idA)
    b, bp = _iarr(idB)
    bufs = [np.zeros(MAX_NAMES, dtype=np.int32) for _ in range(3)]
    cnt = [ctypes.c_int() for _ in range(3)]
    check(lib().gbx_dltc_mul_orders(len(a), ap, len(b), bp, bufs[0].ctypes.data_as(ctypes.c_void_p),
                                    ctypes.byref(cnt[0]), bufs[1].ctypes.data_as(ctypes.c_void_p),
                                    ctypes.byref(cnt[1]), bufs[2].ctypes.data_as(ctypes.c_void_p),
                                    ctypes.byref(cnt[2])))
    return tuple(list(b_[: c.value]) for b_, c in zip(bufs, cnt))


def task_mul(coef, idC, C, idA, A, idB, B, d, lo=None, hi=None, mode="fp64", stream=None):
    """task_mul (DLTC/task.cc:83-137) on whole device tensors C, A, B."""
    c, cp = _iarr(idC)
    a, ap = _iarr(idA)
    b, bp = _iarr(idB)
    l_, lp = _iarr(lo) if lo is not None else (None, None)
    h_, hp = _iarr(hi) if hi is not None else (None, None)
    check(lib().gbx_dltc_task_mul(coef, len(c), cp, _ptr(C), len(a), ap, _ptr(A), len(b), bp, _ptr(B),
                                  ctypes.byref(d), lp, hp, MODES[mode], _stream(stream)))
    return C


def task_sum(coef, idC, C, idA, A, d, lo=None, hi=None, stream=None):
    """task_sum (DLTC/task.cc:51-81) on whole device tensors C, A."""
    c, cp = _iarr(idC)
    a, ap = _iarr(idA)
    l_, lp = _iarr(lo) if lo is not None else (None, None)
    h_, hp = _iarr(hi) if hi is not None else (None, None)
    check(lib().gbx_dltc_task_sum(coef, len(c), cp, _ptr(C), len(a), ap, _ptr(A), ctypes.byref(d), lp, hp,
                                  _stream(stream)))
    return C


def table(which):
    """dict(tensors=[(name, [0 hole / 1 particle per index])], exprs=[dict]) of a residual table."""
    w = TABLES.get(which, which)
    n, nt = ctypes.c_int(0), ctypes.c_int(0)
    check(lib().gbx_dltc_table(w, None, ctypes.byref(n), None, ctypes.byref(nt), None, 0))
    ex = (Expr * n.value)()
    types = np.zeros(5 * nt.value, dtype=np.int32)
    names = ctypes.create_string_buffer(32 * nt.value)
    check(lib().gbx_dltc_table(w, ex, ctypes.byref(n), types.ctypes.data_as(ctypes.c_void_p), ctypes.byref(nt),
                               names, 32))
    tensors = []
    for i in range(nt.value):
        nm = names.raw[32 * i:32 * (i + 1)].split(b"\0", 1)[0].decode()
        r = int(types[5 * i])
        tensors.append((nm, [int(x) for x in types[5 * i + 1:5 * i + 1 + r]]))
    exprs = []
    for e in ex:
        exprs.append(dict(kind=e.kind, index=e.index, layer=e.layer, c=e.c, a=e.a, b=e.b, coef=e.coef,
                          idC=list(e.idc[:e.rc]), idA=list(e.ida[:e.ra]), idB=list(e.idb[:e.rb])))
    return dict(tensors=tensors, exprs=exprs)


class _DevView:
    """A device buffer as a torch tensor (zero copy, CUDA array interface)."""

    def __init__(self, ptr, n):
        self.__cuda_array_interface__ = {"shape": (int(n),), "typestr": "<f8", "data": (int(ptr), False),
                                         "version": 3, "strides": None}


class Program:
    """A residual table bound to zeroed device tensors (gbx_dltc_program)."""

    def __init__(self, which, d, mode="fp64"):
        self.handle = ctypes.c_void_p()
        self.which = TABLES.get(which, which)
        self.d = d
        check(lib().gbx_dltc_program_create(self.which, ctypes.byref(d), MODES[mode], ctypes.byref(self.handle)))
        self.table = table(self.which)

    def tensor(self, t):
        """Tensor t's device buffer as a flat torch view."""
        p, n = ctypes.c_void_p(), ctypes.c_int64()
        check(lib().gbx_dltc_program_tensor(self.handle, t, ctypes.byref(p), ctypes.byref(n)))
        return torch.as_tensor(_DevView(p.value, n.value), device="cuda")

    def run(self, first=0, count=-1, stream=None):
        check(lib().gbx_dltc_program_run(self.handle, first, count, _stream(stream)))

    def check(self):
        check(lib().gbx_dltc_program_check(self.handle))

    @property
    def flops(self):
        return lib().gbx_dltc_program_flops(self.handle)

    def close(self):
        if getattr(self, "handle", None) and self.handle.value:
            lib().gbx_dltc_program_destroy(self.handle)
            self.handle = ctypes.c_void_p()

    def __del__(self):
        self.close()
