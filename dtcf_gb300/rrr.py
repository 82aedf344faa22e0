"""Host-side mirror of RRR's tensor / contraction interface on one process.

``Tensor`` keeps RRR's storage (tensor.h:40-120): the unique blocks of a
symmetric block-distributed tensor, each a dense row-major block of
``block_range`` extents, contiguous on the device, with their block addresses.
``Contraction(A, B, C).contract("a,b,k,l", "m,n,k,l", "a,b,m,n")`` mirrors
Contraction::contract (contraction.h:262) and runs the node-local work through
the C ABI (gbx_plan_create / gbx_execute).
"""
import ctypes

import numpy as np
import torch

from ._lib import lib, check

MODES = {"fp64": 0, "split": 1}


class TensorDesc(ctypes.Structure):
    """gbx_tensor_desc (include/gbx.h)."""
    _fields_ = [("dims", ctypes.c_int), ("sym", ctypes.c_char_p), ("block_range", ctypes.c_void_p),
                ("vgrid", ctypes.c_void_p), ("num_tiles", ctypes.c_int), ("tile_address", ctypes.c_void_p)]


def _stream(stream):
    s = stream if stream is not None else torch.cuda.current_stream()
    return ctypes.c_void_p(s.cuda_stream)


def unique_blocks(sym, vgrid, stream=None):
    """Block addresses RRR stores on one process (Tensor::generate_data /
    isValid, tensor.cc:617-694), generated on the device
    (gbx_rrr_unique_tiles): (num_tiles, dims) int32 CUDA tensor."""
    g = np.ascontiguousarray(vgrid, dtype=np.int32)
    n = ctypes.c_int()
    check(lib().gbx_rrr_unique_tiles(len(sym), sym.encode(), g.ctypes.data_as(ctypes.c_void_p), None, 0,
                                     ctypes.byref(n), _stream(stream)))
    out = torch.zeros((max(1, n.value), len(sym)), dtype=torch.int32, device="cuda")
    check(lib().gbx_rrr_unique_tiles(len(sym), sym.encode(), g.ctypes.data_as(ctypes.c_void_p),
                                     ctypes.c_void_p(out.data_ptr()), n.value, ctypes.byref(n), _stream(stream)))
    return out[: n.value]


class Tensor:
    def __init__(self, sym, size, vgrid, addrs=None, device="cuda"):
        self.sym = sym
        self.size = list(size)
        self.vgrid = list(vgrid)
        self.block_range = [s // v for s, v in zip(size, vgrid)]
        self.block_size = int(np.prod(self.block_range))
        if addrs is None:
            self.d_addrs = unique_blocks(sym, vgrid)
            self.addrs = self.d_addrs.cpu().numpy()
        else:
            self.addrs = np.ascontiguousarray(addrs, dtype=np.int32)
            self.d_addrs = torch.from_numpy(self.addrs.copy()).to(device)
        self.num_tiles = self.addrs.shape[0]
        self.tiles = torch.zeros(self.num_tiles * self.block_size, dtype=torch.float64, device=device)
        self._keep = []

    def initialize(self, stream=None):
        """Tensor::initialize (tensor.cc:315-335) on the device: each block
        holds the constant sum_d sin(block_address_d) (tensor.cc:744-758)."""
        g = np.ascontiguousarray(self.vgrid, dtype=np.int32)
        check(lib().gbx_rrr_initialize(len(self.sym), g.ctypes.data_as(ctypes.c_void_p),
                                       ctypes.c_void_p(self.d_addrs.data_ptr()), self.num_tiles, self.block_size,
                                       ctypes.c_void_p(self.tiles.data_ptr()), _stream(stream)))
        return self

    def desc(self):
        br = np.ascontiguousarray(self.block_range, dtype=np.int32)
        vg = np.ascontiguousarray(self.vgrid, dtype=np.int32)
        sym = self.sym.encode()
        self._keep = [br, vg, sym, self.addrs]
        return TensorDesc(len(self.sym), sym, br.ctypes.data, vg.ctypes.data, self.num_tiles, self.addrs.ctypes.data)


class Plan:
    def __init__(self, A, B, C, idxA, idxB, idxC, mode="fp64", sign=1, slices=6):
        self.handle = ctypes.c_void_p()
        da, db, dc = A.desc(), B.desc(), C.desc()
        check(lib().gbx_plan_create(ctypes.byref(da), ctypes.byref(db), ctypes.byref(dc), idxA.encode(),
                                    idxB.encode(), idxC.encode(), MODES[mode], sign, slices,
                                    ctypes.byref(self.handle)))

    @property
    def flops(self):
        return lib().gbx_plan_flops(self.handle)

    def execute(self, A, B, C, alpha=1.0, stream=None):
        s = stream if stream is not None else torch.cuda.current_stream()
        check(lib().gbx_execute(self.handle, ctypes.c_void_p(A.tiles.data_ptr()), ctypes.c_void_p(B.tiles.data_ptr()),
                                ctypes.c_void_p(C.tiles.data_ptr()), alpha, ctypes.c_void_p(s.cuda_stream)))

    def __del__(self):
        if getattr(self, "handle", None) and self.handle.value:
            lib().gbx_plan_destroy(self.handle)
            self.handle = ctypes.c_void_p()


class Contraction:
    """Contraction(A, B, C).contract(strA, strB, strC): C += alpha * A * B on
    this process's stored C blocks (contraction.cc:2447-2870, node-local part)."""

    def __init__(self, A, B, C, mode="fp64", sign=1, slices=6):
        self.A, self.B, self.C = A, B, C
        self.mode, self.sign, self.slices = mode, sign, slices
        self._plans = {}

    def plan(self, strA, strB, strC):
        key = (strA, strB, strC)
        if key not in self._plans:
            self._plans[key] = Plan(self.A, self.B, self.C, strA, strB, strC, self.mode, self.sign, self.slices)
        return self._plans[key]

    def contract(self, strA, strB, strC, alpha=1.0, stream=None):
        self.plan(strA, strB, strC).execute(self.A, self.B, self.C, alpha, stream)
        return self.C
