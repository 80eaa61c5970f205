"""formoniq_gb300: the Galerkin assembly and Krylov solve path of formoniq on GB300.

The compute lives in the native library ``_lib/libformoniq_gb300.so`` (CUDA
sm_103a kernels behind the C ABI declared in ``include/formoniq_gpu.h``). This
module binds that ABI with ctypes and mirrors the reference's Rust API on the
path, so calling code reads like formoniq:

    mesh = Mesh.kuhn_cube(ctx, 3, 32)            # CartesianGrid::new_unit(3, 32).triangulate()
    mesh.kuhn_lengths(jitter=0.1, seed=7)         # MeshCoords::to_edge_lengths_sq
    wc = WhitneyComplex(mesh)                     # WhitneyComplex::new
    m1 = wc.mass(1)                               # HilbertComplex::mass
    sigma, u, p, rep = solve_source(wc, f, 1)     # elliptic::solve_source

There is no CPU fallback: importing succeeds without the library, but every
entry point raises ``FqUnavailable`` when it is missing, and every compute call
needs a CUDA device.
"""
from __future__ import annotations

import ctypes
import math
import os
import weakref
from dataclasses import dataclass
from typing import Optional

import numpy as np

__all__ = [
    "FQ_MASS", "FQ_DIF_TRIAL", "FQ_DIF_TEST", "FQ_DIF_BOTH", "FQ_ABSOLUTE", "FQ_RELATIVE", "FQ_FP64", "FQ_FP32", "FQ_FP64_IEEE",
    "FqError", "FqUnavailable", "Context", "Mesh", "Matrix", "WhitneyComplex", "MixedProblem", "SolveOpts",
    "Report", "solve_source", "solve_dirac_source", "dirac_system", "minres", "cg", "hx_cg", "hx_apply", "lib_path",
    "load", "exported_symbols", "FQ_PC_AUTO", "FQ_PC_JACOBI", "FQ_PC_HX", "FQ_PC_DIRECT", "FQ_PC_COMPARISON", "Server", "FQ_REQ_HODGE", "FQ_REQ_DIRAC",
    "Batch", "FQ_BATCH_MASS", "FQ_BATCH_HDIF", "ElementOperator", "derham_map", "Leapfrog",
    "source_nodes", "source_form", "SparseLu",
]

FQ_MASS, FQ_DIF_TRIAL, FQ_DIF_TEST, FQ_DIF_BOTH = 0, 1, 2, 3
FQ_ABSOLUTE, FQ_RELATIVE = 0, 1
FQ_FP64, FQ_FP32, FQ_FP64_IEEE = 0, 1, 2
FQ_PC_AUTO, FQ_PC_JACOBI, FQ_PC_HX, FQ_PC_DIRECT, FQ_PC_COMPARISON = 0, 1, 2, 3, 4
FQ_REQ_HODGE, FQ_REQ_DIRAC = 0, 1
FQ_BATCH_MASS, FQ_BATCH_HDIF = 0, 1

_STATUS = {
    0: "FQ_OK", 1: "FQ_INVALID_ARG", 2: "FQ_DEGENERATE_CELL", 3: "FQ_NOT_CONVERGED", 4: "FQ_BREAKDOWN",
    5: "FQ_OOM_BUDGET", 6: "FQ_TIMEOUT", 7: "FQ_CUDA_ERROR", 8: "FQ_NO_DEVICE", 9: "FQ_UNSUPPORTED",
}

_HERE = os.path.dirname(os.path.abspath(__file__))


def lib_path() -> str:
    return os.path.join(_HERE, "_lib", "libformoniq_gb300.so")


class FqUnavailable(RuntimeError):
    """The native library is missing: build it with ``__graft_entry__.build()``."""


class FqError(RuntimeError):
    def __init__(self, status: int, message: str = ""):
        self.status = status
        self.name = _STATUS.get(status, f"status {status}")
        super().__init__(f"{self.name}: {message}" if message else self.name)


class SolveOpts(ctypes.Structure):
    """StopCriterion (iterative/src/lib.rs:193-208) plus refinement knobs."""

    _fields_ = [("rtol", ctypes.c_double), ("max_iters", ctypes.c_int64), ("precision", ctypes.c_int),
                ("refine_rtol", ctypes.c_double), ("max_refinements", ctypes.c_int64),
                ("preconditioner", ctypes.c_int)]

    @staticmethod
    def default(**kw) -> "SolveOpts":
        o = SolveOpts(1e-10, 10_000, FQ_FP64, 1e-12, 6, FQ_PC_AUTO)
        for k, v in kw.items():
            setattr(o, k, v)
        return o


class _Report(ctypes.Structure):
    _fields_ = [("iters", ctypes.c_int64), ("residual", ctypes.c_double), ("converged", ctypes.c_int32),
                ("refinements", ctypes.c_int32), ("true_residual", ctypes.c_double)]


class _Request(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int), ("dim", ctypes.c_int), ("nbox", ctypes.c_int), ("grade", ctypes.c_int),
                ("bc", ctypes.c_int), ("minkowski", ctypes.c_int), ("jitter", ctypes.c_double),
                ("seed", ctypes.c_uint64), ("mass_term", ctypes.c_double), ("arrival_ms", ctypes.c_double),
                ("lengths", ctypes.c_void_p), ("source", ctypes.c_void_p), ("solution", ctypes.c_void_p),
                ("opts", SolveOpts)]


class _Result(ctypes.Structure):
    _fields_ = [("status", ctypes.c_int32), ("lane", ctypes.c_int32), ("report", _Report),
                ("queue_ms", ctypes.c_double), ("run_ms", ctypes.c_double), ("latency_ms", ctypes.c_double),
                ("start_ms", ctypes.c_double), ("end_ms", ctypes.c_double), ("checksum", ctypes.c_double),
                ("ndofs", ctypes.c_uint64), ("cache_hit", ctypes.c_int32), ("pad", ctypes.c_int32)]


class _ServerStats(ctypes.Structure):
    _fields_ = [("submitted", ctypes.c_uint64), ("completed", ctypes.c_uint64), ("cache_hits", ctypes.c_uint64),
                ("evictions", ctypes.c_uint64), ("peak_committed_bytes", ctypes.c_uint64),
                ("resident_bytes", ctypes.c_uint64), ("busy_ms", ctypes.c_double)]


@dataclass
class Report:
    """Report (iterative/src/lib.rs:212-219)."""

    iters: int
    residual: float
    converged: bool
    refinements: int = 0
    true_residual: float = 0.0

    @staticmethod
    def of(r: _Report) -> "Report":
        return Report(int(r.iters), float(r.residual), bool(r.converged), int(r.refinements),
                      float(r.true_residual))


_lib = None

_P = ctypes.c_void_p
_I32P = ctypes.POINTER(ctypes.c_int32)
_I64P = ctypes.POINTER(ctypes.c_int64)
_DP = ctypes.POINTER(ctypes.c_double)

# name -> (restype, argtypes); every function declared in include/formoniq_gpu.h
_SIGNATURES = {
    "fq_ctx_create": (ctypes.c_int, [ctypes.c_int, _P, ctypes.c_uint64, ctypes.POINTER(_P)]),
    "fq_ctx_destroy": (None, [_P]),
    "fq_status_name": (ctypes.c_char_p, [ctypes.c_int]),
    "fq_ctx_last_error": (ctypes.c_char_p, [_P]),
    "fq_ctx_synchronize": (ctypes.c_int, [_P]),
    "fq_ctx_bytes_in_use": (ctypes.c_uint64, [_P]),
    "fq_ctx_kernel_launches": (ctypes.c_uint64, [_P]),
    "fq_default_solve_opts": (None, [ctypes.POINTER(SolveOpts)]),
    "fq_ctx_set_profiling": (ctypes.c_int, [_P, ctypes.c_int]),
    "fq_ctx_set_scatter_shape": (ctypes.c_int, [_P, ctypes.c_int, ctypes.c_int]),
    "fq_ctx_profile": (ctypes.c_int, [_P, _DP, _I64P, ctypes.c_int, ctypes.c_int]),
    "fq_measure_fma_peak": (ctypes.c_int, [_P, ctypes.c_int, _DP]),
    "fq_mesh_from_cells": (ctypes.c_int, [_P, ctypes.c_int, ctypes.c_int64, _I32P, ctypes.POINTER(_P)]),
    "fq_mesh_kuhn_cube": (ctypes.c_int, [_P, ctypes.c_int, ctypes.c_int, ctypes.POINTER(_P)]),
    "fq_mesh_destroy": (None, [_P]),
    "fq_mesh_dim": (ctypes.c_int, [_P]),
    "fq_mesh_nsimplices": (ctypes.c_int64, [_P, ctypes.c_int]),
    "fq_mesh_ndofs": (ctypes.c_int64, [_P, ctypes.c_int, ctypes.c_int]),
    "fq_mesh_simplices": (ctypes.c_int, [_P, ctypes.c_int, _I32P]),
    "fq_mesh_interior": (ctypes.c_int, [_P, ctypes.c_int, _I64P]),
    "fq_mesh_orientation": (ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_int8)]),
    "fq_mesh_set_lengths_sq": (ctypes.c_int, [_P, _DP, ctypes.c_int]),
    "fq_mesh_get_lengths_sq": (ctypes.c_int, [_P, _DP]),
    "fq_mesh_lengths_from_coords": (ctypes.c_int, [_P, _DP, ctypes.c_int, _DP]),
    "fq_mesh_kuhn_lengths": (ctypes.c_int, [_P, _DP, _DP, ctypes.c_double, ctypes.c_uint64]),
    "fq_cell_metrics": (ctypes.c_int, [_P, _P, _P, _P, _P]),
    "fq_element_matrices": (ctypes.c_int, [_P, _P, ctypes.c_int, ctypes.c_int, ctypes.c_int, _P,
                                           ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)]),
    "fq_assemble": (ctypes.c_int, [_P, _P, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                   ctypes.POINTER(_P)]),
    "fq_reassemble": (ctypes.c_int, [_P, _P, _P]),
    "fq_reassemble_many": (ctypes.c_int, [_P, ctypes.POINTER(_P), ctypes.c_int]),
    "fq_elemop_create": (ctypes.c_int, [_P, _P, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.POINTER(_P)]),
    "fq_elemop_info": (ctypes.c_int, [_P, _I64P, _I64P]),
    "fq_elemop_apply": (ctypes.c_int, [_P, _P, _P]),
    "fq_elemop_diagonal": (ctypes.c_int, [_P, _P]),
    "fq_elemop_cg": (ctypes.c_int, [_P, _P, _P, _P, ctypes.POINTER(SolveOpts), ctypes.POINTER(_Report)]),
    "fq_elemop_destroy": (None, [_P]),
    "fq_derham_npoints": (ctypes.c_int, [ctypes.c_int, ctypes.c_int]),
    "fq_source_npoints": (ctypes.c_int, [ctypes.c_int, ctypes.c_int]),
    "fq_source_nodes": (ctypes.c_int, [_P, _P, _P, ctypes.c_int, ctypes.c_int, _P]),
    "fq_source_assemble": (ctypes.c_int, [_P, _P, ctypes.c_int, ctypes.c_int, ctypes.c_int, _P, ctypes.c_int, _P,
                                          _P]),
    "fq_leapfrog_create": (ctypes.c_int, [_P, _P, ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.POINTER(_P)]),
    "fq_leapfrog_info": (ctypes.c_int, [_P, _I64P, _I64P, _I64P]),
    "fq_leapfrog_step": (ctypes.c_int, [_P, _P, ctypes.c_int64]),
    "fq_leapfrog_energy": (ctypes.c_int, [_P, _P, _DP, _DP]),
    "fq_leapfrog_destroy": (None, [_P]),
    "fq_derham_nodes": (ctypes.c_int, [_P, _P, _P, ctypes.c_int, ctypes.c_int, ctypes.c_int, _P]),
    "fq_derham_reduce": (ctypes.c_int, [_P, _P, _P, ctypes.c_int, ctypes.c_int, ctypes.c_int, _P, _P]),
    "fq_hdif_gram": (ctypes.c_int, [_P, _P, ctypes.c_int, ctypes.c_int, ctypes.POINTER(_P)]),
    "fq_coboundary": (ctypes.c_int, [_P, _P, ctypes.c_int, ctypes.c_int, ctypes.POINTER(_P)]),
    "fq_assemble_host": (ctypes.c_int, [_P, _P, _P, _DP, _P]),
    "fq_assemble_host_many": (ctypes.c_int, [_P, _P, _DP, ctypes.POINTER(_P), ctypes.POINTER(_P), ctypes.c_int]),
    "fq_reassemble_noalloc": (ctypes.c_int, [_P, _P, _P, _P]),
    "fq_matrix_info": (ctypes.c_int, [_P, _I64P, _I64P, _I64P, ctypes.POINTER(ctypes.c_int)]),
    "fq_matrix_scatter_bytes": (ctypes.c_int, [_P, _I64P]),
    "fq_matrix_device_arrays": (ctypes.c_int, [_P, ctypes.POINTER(_P), ctypes.POINTER(_P), ctypes.POINTER(_P)]),
    "fq_matrix_copy_to_host": (ctypes.c_int, [_P, _P, _I32P, _I32P, _P]),
    "fq_matrix_destroy": (None, [_P]),
    "fq_spmv": (ctypes.c_int, [_P, _P, _P, _P]),
    "fq_minres": (ctypes.c_int, [_P, _P, _P, _P, _P, ctypes.POINTER(SolveOpts), ctypes.POINTER(_Report)]),
    "fq_cg": (ctypes.c_int, [_P, _P, _P, _P, _P, ctypes.POINTER(SolveOpts), ctypes.POINTER(_Report)]),
    "fq_hx_cg": (ctypes.c_int, [_P, _P, ctypes.c_int, ctypes.c_int, _DP, _DP, ctypes.POINTER(SolveOpts),
                                ctypes.POINTER(_Report)]),
    "fq_hx_apply": (ctypes.c_int, [_P, _P, ctypes.c_int, ctypes.c_int, _DP, _DP]),
    "fq_batch_create": (ctypes.c_int, [_P, ctypes.c_int, ctypes.POINTER(_P), _I32P, ctypes.c_int, ctypes.POINTER(_P)]),
    "fq_batch_tune": (ctypes.c_int, [_P, ctypes.c_int]),
    "fq_batch_set_launch": (ctypes.c_int, [_P, ctypes.c_int, ctypes.c_int, ctypes.c_int]),
    "fq_batch_set_element_launch": (ctypes.c_int, [_P, ctypes.c_int, ctypes.c_int]),
    "fq_batch_fused_registers": (ctypes.c_int, []),
    "fq_batch_assemble": (ctypes.c_int, [_P, ctypes.c_int]),
    "fq_batch_assemble_per_mesh": (ctypes.c_int, [_P, ctypes.c_int]),
    "fq_batch_info": (ctypes.c_int, [_P, _I64P, _I64P, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)]),
    "fq_batch_launch_config": (ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int),
                                              ctypes.POINTER(ctypes.c_int), ctypes.c_int]),
    "fq_batch_matrix": (ctypes.c_int, [_P, ctypes.c_int, _I64P, _I64P, ctypes.POINTER(_P), ctypes.POINTER(_P),
                                       ctypes.POINTER(_P)]),
    "fq_batch_copy_to_host": (ctypes.c_int, [_P, ctypes.c_int, _I32P, _I32P, _DP]),
    "fq_batch_destroy": (None, [_P]),
    "fq_server_create": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_uint64, ctypes.c_int, ctypes.POINTER(_P)]),
    "fq_server_submit": (ctypes.c_int, [_P, ctypes.POINTER(_Request), ctypes.POINTER(ctypes.c_uint64)]),
    "fq_server_wait": (ctypes.c_int, [_P, ctypes.c_uint64, ctypes.POINTER(_Result)]),
    "fq_server_get_stats": (ctypes.c_int, [_P, ctypes.POINTER(_ServerStats)]),
    "fq_server_destroy": (None, [_P]),
    "fq_mixed_create": (ctypes.c_int, [_P, _P, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.POINTER(_P)]),
    "fq_mixed_reassemble": (ctypes.c_int, [_P]),
    "fq_mixed_solve": (ctypes.c_int, [_P, _DP, _DP, _DP, _DP, ctypes.POINTER(SolveOpts), ctypes.POINTER(_Report)]),
    "fq_mixed_solve_device": (ctypes.c_int, [_P, _P, _P, _P, _P, ctypes.POINTER(SolveOpts),
                                             ctypes.POINTER(_Report)]),
    "fq_mixed_info": (ctypes.c_int, [_P, _I64P, _I64P, _I64P, _I64P]),
    "fq_mixed_system": (_P, [_P]),
    "fq_mixed_destroy": (None, [_P]),
    "fq_solve_source": (ctypes.c_int, [_P, _P, ctypes.c_int, ctypes.c_int, _DP, _DP, _DP, _DP,
                                       ctypes.POINTER(SolveOpts), ctypes.POINTER(_Report)]),
    "fq_solve_dirac_source": (ctypes.c_int, [_P, _P, ctypes.c_double, _DP, _DP, _DP, ctypes.POINTER(SolveOpts),
                                             ctypes.POINTER(_Report)]),
    "fq_dirac_system": (ctypes.c_int, [_P, _P, ctypes.c_double, ctypes.POINTER(_P)]),
    "fq_sparse_lu_create": (ctypes.c_int, [_P, _P, _P, ctypes.POINTER(_P)]),
    "fq_sparse_lu_factor": (ctypes.c_int, [_P, _P, ctypes.c_int]),
    "fq_sparse_lu_solve": (ctypes.c_int, [_P, _P, _P, _P, ctypes.POINTER(SolveOpts), ctypes.POINTER(_Report)]),
    "fq_sparse_lu_info": (ctypes.c_int, [_P, _I64P, _I64P, _DP, _I64P, _I64P]),
    "fq_sparse_lu_destroy": (None, [_P]),
    "fq_sparse_lu_analyse_host": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int64, _I32P, _I32P, _I32P, _DP]),
}


def exported_symbols():
    return list(_SIGNATURES)


def load():
    """Load the native library (raises FqUnavailable when it is not built)."""
    global _lib
    if _lib is None:
        path = lib_path()
        if not os.path.exists(path):
            raise FqUnavailable(f"{path} is missing; build it with __graft_entry__.build()")
        L = ctypes.CDLL(path)
        for name, (res, args) in _SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _dp(a: np.ndarray):
    return a.ctypes.data_as(_DP)


class Context:
    """fq_ctx: a device, a CUDA stream and an HBM budget (0 = unlimited)."""

    def __init__(self, device: int = 0, stream: int = 0, budget_bytes: int = 0):
        L = load()
        h = _P()
        s = L.fq_ctx_create(device, _P(stream) if stream else None, budget_bytes, ctypes.byref(h))
        if s != 0:
            raise FqError(s, "fq_ctx_create")
        self.h = h
        self.L = L
        self.device = device
        # native objects made on this context, closed before it (the C ABI needs
        # meshes, matrices and problems destroyed before their context)
        self._children = weakref.WeakSet()
        self._meshes = weakref.WeakSet()

    def _adopt(self, obj, mesh: bool = False):
        (self._meshes if mesh else self._children).add(obj)
        return obj

    def check(self, status: int, what: str = ""):
        if status != 0:
            msg = self.L.fq_ctx_last_error(self.h)
            raise FqError(status, f"{what}: {msg.decode() if msg else ''}")

    def synchronize(self):
        self.check(self.L.fq_ctx_synchronize(self.h), "synchronize")

    @property
    def bytes_in_use(self) -> int:
        return int(self.L.fq_ctx_bytes_in_use(self.h))

    @property
    def kernel_launches(self) -> int:
        return int(self.L.fq_ctx_kernel_launches(self.h))

    def set_profiling(self, enable: bool):
        self.check(self.L.fq_ctx_set_profiling(self.h, int(enable)), "fq_ctx_set_profiling")

    def set_scatter_shape(self, slots_per_thread: int, blocks_per_sm: int = 0):
        """Launch shape of the symmetric scatter (fq_ctx_set_scatter_shape)."""
        self.check(self.L.fq_ctx_set_scatter_shape(self.h, int(slots_per_thread), int(blocks_per_sm)),
                   "fq_ctx_set_scatter_shape")

    def profile(self, reset: bool = False):
        """(element_ms, scatter_ms), (element_launches, scatter_launches)."""
        ms = (ctypes.c_double * 4)()
        n = (ctypes.c_int64 * 4)()
        self.check(self.L.fq_ctx_profile(self.h, ms, n, 4, int(reset)))
        return list(ms)[:2], list(n)[:2]

    def fma_peak_tflops(self, fp64: bool = True) -> float:
        t = ctypes.c_double()
        self.check(self.L.fq_measure_fma_peak(self.h, int(fp64), ctypes.byref(t)), "fq_measure_fma_peak")
        return t.value

    def close(self):
        if getattr(self, "h", None):
            for group in (self._children, self._meshes):
                for obj in list(group):
                    try:
                        obj.close()
                    except Exception:
                        pass
            self.L.fq_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Matrix:
    """An assembled Galerkin matrix resident on the device (GalerkinMatrix = CsrMatrix)."""

    def __init__(self, ctx: Context, h, owned: bool = True):
        self.ctx, self.h, self.owned = ctx, h, owned
        if owned:
            ctx._adopt(self)

    def info(self):
        nr, nc, nnz, pr = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int()
        self.ctx.check(self.ctx.L.fq_matrix_info(self.h, ctypes.byref(nr), ctypes.byref(nc), ctypes.byref(nnz),
                                                 ctypes.byref(pr)))
        return nr.value, nc.value, nnz.value, pr.value

    @property
    def shape(self):
        nr, nc, _, _ = self.info()
        return (nr, nc)

    @property
    def nnz(self) -> int:
        return self.info()[2]

    def scatter_bytes(self) -> int:
        """Bytes one re-assembly's scatter reads and writes for this matrix (fq_matrix_scatter_bytes)."""
        b = ctypes.c_int64()
        self.ctx.check(self.ctx.L.fq_matrix_scatter_bytes(self.h, ctypes.byref(b)), "fq_matrix_scatter_bytes")
        return b.value

    def host_arrays(self):
        nr, nc, nnz, pr = self.info()
        rp = np.zeros(nr + 1, np.int32)
        ci = np.zeros(max(nnz, 1), np.int32)
        vv = np.zeros(max(nnz, 1), np.float32 if pr == FQ_FP32 else np.float64)
        self.ctx.check(self.ctx.L.fq_matrix_copy_to_host(self.ctx.h, self.h, rp.ctypes.data_as(_I32P),
                                                         ci.ctypes.data_as(_I32P), vv.ctypes.data_as(_P)))
        return rp, ci[:nnz], vv[:nnz]

    def to_scipy(self):
        import scipy.sparse as sp

        nr, nc, _, _ = self.info()
        rp, ci, vv = self.host_arrays()
        m = sp.csr_matrix((vv, ci, rp), shape=(nr, nc))
        m.has_sorted_indices = True
        return m

    def device_arrays(self):
        rp, ci, vv = _P(), _P(), _P()
        self.ctx.check(self.ctx.L.fq_matrix_device_arrays(self.h, ctypes.byref(rp), ctypes.byref(ci),
                                                          ctypes.byref(vv)))
        return rp.value, ci.value, vv.value

    def reassemble(self, mesh: "Mesh"):
        self.ctx.check(self.ctx.L.fq_reassemble(self.ctx.h, mesh.h, self.h), "fq_reassemble")

    @staticmethod
    def reassemble_many(mats):
        """fq_reassemble_many: re-assemble every matrix (of one context) with one
        status read at the end."""
        mats = list(mats)
        if not mats:
            return
        ctx = mats[0].ctx
        arr = (_P * len(mats))(*[m.h for m in mats])
        ctx.check(ctx.L.fq_reassemble_many(ctx.h, arr, len(mats)), "fq_reassemble_many")

    def reassemble_noalloc(self, mesh: "Mesh", values_ptr: int):
        """Values of this matrix's pattern into a caller-owned device buffer,
        with no device allocation (see fq_reassemble_noalloc)."""
        self.ctx.check(self.ctx.L.fq_reassemble_noalloc(self.ctx.h, mesh.h, self.h, _P(values_ptr)),
                       "fq_reassemble_noalloc")

    def close(self):
        if self.owned and getattr(self, "h", None):
            self.ctx.L.fq_matrix_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Mesh:
    """A simplicial complex with Regge geometry: Complex + MeshLengthsSq."""

    def __init__(self, ctx: Context, h):
        self.ctx, self.h = ctx, h
        ctx._adopt(self, mesh=True)

    @staticmethod
    def from_cells(ctx: Context, cells: np.ndarray) -> "Mesh":
        cells = np.ascontiguousarray(cells, np.int32)
        h = _P()
        ctx.check(ctx.L.fq_mesh_from_cells(ctx.h, cells.shape[1] - 1, cells.shape[0], cells.ctypes.data_as(_I32P),
                                           ctypes.byref(h)), "fq_mesh_from_cells")
        return Mesh(ctx, h)

    @staticmethod
    def kuhn_cube(ctx: Context, dim: int, nboxes: int) -> "Mesh":
        h = _P()
        ctx.check(ctx.L.fq_mesh_kuhn_cube(ctx.h, dim, nboxes, ctypes.byref(h)), "fq_mesh_kuhn_cube")
        return Mesh(ctx, h)

    @property
    def dim(self) -> int:
        return self.ctx.L.fq_mesh_dim(self.h)

    def nsimplices(self, k: int) -> int:
        return int(self.ctx.L.fq_mesh_nsimplices(self.h, k))

    def ncells(self) -> int:
        return self.nsimplices(self.dim)

    def ndofs(self, k: int, bc: int = FQ_ABSOLUTE) -> int:
        return int(self.ctx.L.fq_mesh_ndofs(self.h, k, bc))

    def simplices(self, k: int) -> np.ndarray:
        out = np.zeros((self.nsimplices(k), k + 1), np.int32)
        self.ctx.check(self.ctx.L.fq_mesh_simplices(self.h, k, out.ctypes.data_as(_I32P)))
        return out

    def interior(self, k: int) -> np.ndarray:
        out = np.zeros(max(self.ndofs(k, FQ_RELATIVE), 1), np.int64)
        self.ctx.check(self.ctx.L.fq_mesh_interior(self.h, k, out.ctypes.data_as(_I64P)))
        return out[: self.ndofs(k, FQ_RELATIVE)]

    def orientation(self) -> np.ndarray:
        out = np.zeros(self.ncells(), np.int8)
        self.ctx.check(self.ctx.L.fq_mesh_orientation(self.h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_int8))))
        return out

    def set_lengths_sq(self, lengths: np.ndarray):
        lengths = np.ascontiguousarray(lengths, np.float64)
        self.ctx.check(self.ctx.L.fq_mesh_set_lengths_sq(self.h, _dp(lengths), 0), "fq_mesh_set_lengths_sq")

    def lengths_sq(self) -> np.ndarray:
        out = np.zeros(max(self.nsimplices(1), 1))
        self.ctx.check(self.ctx.L.fq_mesh_get_lengths_sq(self.h, _dp(out)))
        return out[: self.nsimplices(1)]

    def lengths_from_coords(self, coords: np.ndarray, ambient_signs=None):
        coords = np.ascontiguousarray(coords, np.float64)
        signs = None if ambient_signs is None else np.ascontiguousarray(ambient_signs, np.float64)
        self.ctx.check(self.ctx.L.fq_mesh_lengths_from_coords(self.h, _dp(coords), coords.shape[1],
                                                              _dp(signs) if signs is not None else None))

    def kuhn_lengths(self, side=None, ambient_signs=None, jitter: float = 0.0, seed: int = 0):
        side = None if side is None else np.ascontiguousarray(side, np.float64)
        signs = None if ambient_signs is None else np.ascontiguousarray(ambient_signs, np.float64)
        self.ctx.check(self.ctx.L.fq_mesh_kuhn_lengths(self.h, _dp(side) if side is not None else None,
                                                       _dp(signs) if signs is not None else None, float(jitter),
                                                       int(seed)), "fq_mesh_kuhn_lengths")

    def close(self):
        if getattr(self, "h", None):
            self.ctx.L.fq_mesh_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class WhitneyComplex:
    """HilbertComplex (whitney_complex.rs:55-277) on the device: the full
    complex, or the relative one (``relative=True``, essential BC)."""

    def __init__(self, mesh: Mesh, relative: bool = False, precision: int = FQ_FP64):
        self.mesh = mesh
        self.ctx = mesh.ctx
        self.bc = FQ_RELATIVE if relative else FQ_ABSOLUTE
        self.precision = precision

    @property
    def dim(self) -> int:
        return self.mesh.dim

    def relative(self) -> "WhitneyComplex":
        return WhitneyComplex(self.mesh, True, self.precision)

    def ndofs(self, k: int) -> int:
        return self.mesh.ndofs(k, self.bc)

    def _assemble(self, form: int, k: int) -> Matrix:
        h = _P()
        self.ctx.check(self.ctx.L.fq_assemble(self.ctx.h, self.mesh.h, form, k, self.bc, self.precision,
                                              ctypes.byref(h)), "fq_assemble")
        return Matrix(self.ctx, h)

    def mass(self, k: int) -> Matrix:
        return self._assemble(FQ_MASS, k)

    def dif_trial(self, k: int) -> Matrix:
        return self._assemble(FQ_DIF_TRIAL, k)

    def dif_test(self, k: int) -> Matrix:
        return self._assemble(FQ_DIF_TEST, k)

    def dif_both(self, k: int) -> Matrix:
        return self._assemble(FQ_DIF_BOTH, k)

    def hdif_gram(self, k: int) -> Matrix:
        h = _P()
        self.ctx.check(self.ctx.L.fq_hdif_gram(self.ctx.h, self.mesh.h, k, self.bc, ctypes.byref(h)), "fq_hdif_gram")
        return Matrix(self.ctx, h)

    def dif(self, k: int) -> Matrix:
        h = _P()
        self.ctx.check(self.ctx.L.fq_coboundary(self.ctx.h, self.mesh.h, k, self.bc, ctypes.byref(h)),
                       "fq_coboundary")
        return Matrix(self.ctx, h)


class MixedProblem:
    """The resident mixed Hodge-Laplace system of elliptic::solve_source."""

    def __init__(self, mesh: Mesh, grade: int, bc: int = FQ_ABSOLUTE, precision: int = FQ_FP64):
        self.mesh, self.ctx, self.grade, self.bc = mesh, mesh.ctx, grade, bc
        h = _P()
        self.ctx.check(self.ctx.L.fq_mixed_create(self.ctx.h, mesh.h, grade, bc, precision, ctypes.byref(h)),
                       "fq_mixed_create")
        self.h = h
        self.ctx._adopt(self)

    def info(self):
        a, b, c, d = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        self.ctx.check(self.ctx.L.fq_mixed_info(self.h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c),
                                                ctypes.byref(d)))
        return a.value, b.value, c.value, d.value

    def system(self) -> Matrix:
        return Matrix(self.ctx, self.ctx.L.fq_mixed_system(self.h), owned=False)

    def reassemble(self):
        self.ctx.check(self.ctx.L.fq_mixed_reassemble(self.h), "fq_mixed_reassemble")

    def solve(self, source: np.ndarray, opts: Optional[SolveOpts] = None, allow_unconverged=False):
        m = self.mesh
        source = np.ascontiguousarray(source, np.float64)
        nk = m.nsimplices(self.grade)
        nkm = m.nsimplices(self.grade - 1) if self.grade >= 1 else 0
        ns, nu, nh, _ = self.info()
        sigma = np.zeros(max(nkm, 1))
        u = np.zeros(max(nk, 1))
        p = np.zeros(max(nh, 1))
        rep = _Report()
        opts = opts or SolveOpts.default()
        s = self.ctx.L.fq_mixed_solve(self.h, _dp(source), _dp(sigma), _dp(u), _dp(p), ctypes.byref(opts),
                                      ctypes.byref(rep))
        if not (s == 0 or (s == 3 and allow_unconverged)):
            self.ctx.check(s, "fq_mixed_solve")
        return sigma[:nkm], u[:nk], p[:nh], Report.of(rep)

    def solve_device(self, src_ptr: int, sigma_ptr: int, u_ptr: int, p_ptr: int, opts: Optional[SolveOpts] = None):
        rep = _Report()
        opts = opts or SolveOpts.default()
        s = self.ctx.L.fq_mixed_solve_device(self.h, _P(src_ptr), _P(sigma_ptr) if sigma_ptr else None,
                                             _P(u_ptr) if u_ptr else None, _P(p_ptr) if p_ptr else None,
                                             ctypes.byref(opts), ctypes.byref(rep))
        if s not in (0, 3):
            self.ctx.check(s, "fq_mixed_solve_device")
        return Report.of(rep)

    def close(self):
        if getattr(self, "h", None):
            self.ctx.L.fq_mixed_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def solve_source(complex_: WhitneyComplex, source: np.ndarray, grade: int, opts: Optional[SolveOpts] = None,
                 precision: int = FQ_FP64):
    """elliptic::solve_source (problems/elliptic.rs:132-182): (sigma, u, p, report)."""
    prob = MixedProblem(complex_.mesh, grade, complex_.bc, precision)
    try:
        o = opts or SolveOpts.default(precision=precision)
        return prob.solve(source, o)
    finally:
        prob.close()


def solve_dirac_source(mesh: Mesh, mass_term: float, load_: np.ndarray, lift: Optional[np.ndarray] = None,
                       opts: Optional[SolveOpts] = None):
    """dirac::solve_dirac_source (problems/dirac.rs:473-531): the sparse direct
    route (FP64 GMRES on the system's LU, bordered at m = 0) on Kuhn cube
    meshes, MINRES on other meshes or with the MINRES preconditioners."""
    ctx = mesh.ctx
    load_ = np.ascontiguousarray(load_, np.float64)
    lift_a = None if lift is None else np.ascontiguousarray(lift, np.float64)
    x = np.zeros_like(load_)
    rep = _Report()
    opts = opts or SolveOpts.default()
    s = ctx.L.fq_solve_dirac_source(ctx.h, mesh.h, float(mass_term), _dp(load_),
                                    _dp(lift_a) if lift_a is not None else None, _dp(x), ctypes.byref(opts),
                                    ctypes.byref(rep))
    if s not in (0, 3):
        ctx.check(s, "fq_solve_dirac_source")
    return x, Report.of(rep)


class ElementOperator:
    """matfree::ElementOperator: a Whitney pairing applied without assembly.
    Vectors are device pointers (apply, diagonal, cg) or numpy arrays
    (apply_host)."""

    def __init__(self, mesh: Mesh, form: int, grade: int, bc: int = FQ_ABSOLUTE):
        self.ctx, self.mesh = mesh.ctx, mesh
        h = _P()
        self.ctx.check(self.ctx.L.fq_elemop_create(self.ctx.h, mesh.h, form, grade, bc, ctypes.byref(h)),
                       "fq_elemop_create")
        self.h = h
        self.ctx._adopt(self)

    @property
    def shape(self):
        nr, nc = ctypes.c_int64(), ctypes.c_int64()
        self.ctx.check(self.ctx.L.fq_elemop_info(self.h, ctypes.byref(nr), ctypes.byref(nc)))
        return nr.value, nc.value

    def apply(self, x_ptr: int, y_ptr: int):
        self.ctx.check(self.ctx.L.fq_elemop_apply(self.h, _P(x_ptr), _P(y_ptr)), "fq_elemop_apply")

    def diagonal(self, d_ptr: int):
        self.ctx.check(self.ctx.L.fq_elemop_diagonal(self.h, _P(d_ptr)), "fq_elemop_diagonal")

    def cg(self, b_ptr: int, x_ptr: int, inv_diag_ptr: int = 0, opts: Optional[SolveOpts] = None) -> "Report":
        rep = _Report()
        opts = opts or SolveOpts.default()
        s = self.ctx.L.fq_elemop_cg(self.h, _P(b_ptr), _P(x_ptr), _P(inv_diag_ptr) if inv_diag_ptr else None,
                                    ctypes.byref(opts), ctypes.byref(rep))
        if s not in (0, 3):
            self.ctx.check(s, "fq_elemop_cg")
        return Report.of(rep)

    def close(self):
        if getattr(self, "h", None):
            self.ctx.L.fq_elemop_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Leapfrog:
    """solve_dirac_leapfrog / time::Leapfrog on the device: y is a torch CUDA
    float64 tensor in the complex's DOFs, flat by grade (offsets())."""

    def __init__(self, mesh: Mesh, bc: int, dt: float, mass_rtol: float = 0.0):
        self.ctx, self.mesh = mesh.ctx, mesh
        h = _P()
        self.ctx.check(self.ctx.L.fq_leapfrog_create(self.ctx.h, mesh.h, bc, float(dt), float(mass_rtol),
                                                     ctypes.byref(h)), "fq_leapfrog_create")
        self.h = h
        self.ctx._adopt(self)

    def offsets(self):
        n = self.mesh.dim
        off = np.zeros(n + 2, np.int64)
        self.ctx.check(self.ctx.L.fq_leapfrog_info(self.h, None, off.ctypes.data_as(_I64P), None))
        return off

    @property
    def inner_iters(self) -> int:
        it = ctypes.c_int64()
        self.ctx.check(self.ctx.L.fq_leapfrog_info(self.h, None, None, ctypes.byref(it)))
        return it.value

    def step(self, y, nsteps: int = 1):
        import torch

        torch.cuda.synchronize()
        self.ctx.check(self.ctx.L.fq_leapfrog_step(self.h, _P(y.data_ptr()), int(nsteps)), "fq_leapfrog_step")

    def energy(self, y):
        """(1/2 u^T M u, the leapfrog's conserved staggered energy)."""
        import torch

        torch.cuda.synchronize()
        e, c = ctypes.c_double(), ctypes.c_double()
        self.ctx.check(self.ctx.L.fq_leapfrog_energy(self.h, _P(y.data_ptr()), ctypes.byref(e), ctypes.byref(c)),
                       "fq_leapfrog_energy")
        return e.value, c.value

    def close(self):
        if getattr(self, "h", None):
            self.ctx.L.fq_leapfrog_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def derham_map(mesh: Mesh, coords, grade: int, field, degree: int = 3):
    """derham::derham_map (derham/src/project.rs:53-96) on the device.

    coords: torch CUDA tensor [N_0, adim] (float64). field: a callable taking
    the quadrature nodes as a torch CUDA tensor [m, adim] and returning the form's
    components [m, C(adim, grade)] on dx^I (I colex). Returns the cochain as a
    torch CUDA tensor [N_grade]."""
    import math

    import torch

    ctx = mesh.ctx
    coords = coords.to(torch.float64).contiguous()
    adim = coords.shape[1]
    nq = ctx.L.fq_derham_npoints(grade, degree)
    ns = mesh.nsimplices(grade)
    nodes = torch.empty((ns * nq, adim), dtype=torch.float64, device=coords.device)
    torch.cuda.synchronize()
    ctx.check(ctx.L.fq_derham_nodes(ctx.h, mesh.h, _P(coords.data_ptr()), adim, grade, degree,
                                    _P(nodes.data_ptr())), "fq_derham_nodes")
    vals = field(nodes).to(torch.float64).reshape(ns * nq, math.comb(adim, grade)).contiguous()
    out = torch.empty(ns, dtype=torch.float64, device=coords.device)
    torch.cuda.synchronize()
    ctx.check(ctx.L.fq_derham_reduce(ctx.h, mesh.h, _P(coords.data_ptr()), adim, grade, degree,
                                     _P(vals.data_ptr()), _P(out.data_ptr())), "fq_derham_reduce")
    return out


def source_nodes(mesh: Mesh, degree: int = 1, coords=None):
    """The quadrature nodes of the source load (CellQuadrature, formoniq/src/operators.rs:222-261).

    coords None: the barycentric nodes [nq, n+1] shared by every cell; coords a
    torch CUDA tensor [N_0, adim]: the ambient nodes [ncells, nq, adim]."""
    import torch

    ctx = mesh.ctx
    n = mesh.dim
    nq = ctx.L.fq_source_npoints(n, degree)
    if nq <= 0:
        raise FqError(1, f"no quadrature rule of degree {degree} on the {n}-simplex")
    dev = torch.device("cuda", ctx.device)
    if coords is None:
        out = torch.empty((nq, n + 1), dtype=torch.float64, device=dev)
        cptr, adim = None, 0
    else:
        coords = coords.to(torch.float64).contiguous()
        adim = coords.shape[1]
        out = torch.empty((mesh.ncells(), nq, adim), dtype=torch.float64, device=coords.device)
        cptr = _P(coords.data_ptr())
    torch.cuda.synchronize()
    ctx.check(ctx.L.fq_source_nodes(ctx.h, mesh.h, cptr, adim, degree, _P(out.data_ptr())), "fq_source_nodes")
    return out


def source_form(mesh: Mesh, grade: int, values, degree: int = 1, coords=None, bc: int = FQ_ABSOLUTE):
    """SourceForm::new(source, qr).assemble(topology, lengths) on the device
    (formoniq/src/operators.rs:598-635, galerkin.rs:279-312).

    values: a torch CUDA tensor [ncells, nq, ncomp], or a callable taking
    ``source_nodes(mesh, degree, coords)`` and returning it. With coords None
    the components are the section's in each cell's reference frame (ncomp =
    C(n, grade), on dxi^J with xi_j = lambda_{j+1}); with coords [N_0, adim]
    they are a flat ambient form's on dx^A (ncomp = C(adim, grade)), pulled back
    cell by cell. Returns the Galerkin vector [ndofs(grade, bc)] as a torch CUDA
    tensor (FQ_RELATIVE: the interior entries)."""
    import torch

    ctx = mesh.ctx
    if coords is not None:
        coords = coords.to(torch.float64).contiguous()
    adim = 0 if coords is None else coords.shape[1]
    if callable(values):
        values = values(source_nodes(mesh, degree, coords))
    values = values.to(torch.float64).contiguous()
    nq = ctx.L.fq_source_npoints(mesh.dim, degree)
    ncomp = math.comb(adim if coords is not None else mesh.dim, grade)
    if values.numel() != mesh.ncells() * nq * ncomp:
        raise FqError(1, f"values must hold [ncells={mesh.ncells()}, nq={nq}, ncomp={ncomp}] entries")
    out = torch.empty(mesh.ndofs(grade, bc), dtype=torch.float64, device=values.device)
    torch.cuda.synchronize()
    ctx.check(ctx.L.fq_source_assemble(ctx.h, mesh.h, grade, bc, degree,
                                       None if coords is None else _P(coords.data_ptr()), adim,
                                       _P(values.data_ptr()), _P(out.data_ptr())), "fq_source_assemble")
    return out


def dirac_system(mesh: Mesh, mass_term: float) -> Matrix:
    h = _P()
    mesh.ctx.check(mesh.ctx.L.fq_dirac_system(mesh.ctx.h, mesh.h, float(mass_term), ctypes.byref(h)),
                   "fq_dirac_system")
    return Matrix(mesh.ctx, h)


class SparseLu:
    """The sparse direct solver (fq_sparse_lu_*), the stand-in for FaerLu
    (formoniq/src/linalg/faer.rs:51-74): multifrontal LU on a nested-dissection
    ordering of the Kuhn lattice, its factors preconditioning FP64 GMRES.
    ``a`` is an assembled square FP64 matrix of a Kuhn cube mesh."""

    def __init__(self, mesh: Mesh, a: Matrix):
        self.ctx, self.mesh, self.a = mesh.ctx, mesh, a
        h = _P()
        self.ctx.check(self.ctx.L.fq_sparse_lu_create(self.ctx.h, mesh.h, a.h, ctypes.byref(h)), "fq_sparse_lu_create")
        self.h = h
        self.ctx._adopt(self)

    def factor(self, precision: int = FQ_FP32):
        self.ctx.check(self.ctx.L.fq_sparse_lu_factor(self.h, self.a.h, int(precision)), "fq_sparse_lu_factor")
        return self

    def solve_device(self, b_ptr: int, x_ptr: int, opts: Optional[SolveOpts] = None) -> "Report":
        rep = _Report()
        opts = opts or SolveOpts.default()
        s = self.ctx.L.fq_sparse_lu_solve(self.h, self.a.h, _P(b_ptr), _P(x_ptr), ctypes.byref(opts), ctypes.byref(rep))
        if s not in (0, 3):
            self.ctx.check(s, "fq_sparse_lu_solve")
        return Report.of(rep)

    def solve(self, b: np.ndarray, opts: Optional[SolveOpts] = None):
        import torch

        bd = torch.tensor(np.ascontiguousarray(b, np.float64), device="cuda")
        xd = torch.empty_like(bd)
        torch.cuda.synchronize()
        rep = self.solve_device(bd.data_ptr(), xd.data_ptr(), opts)
        return xd.cpu().numpy(), rep

    def info(self) -> dict:
        fr, lv, fb, pp = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        fl = ctypes.c_double()
        self.ctx.check(self.ctx.L.fq_sparse_lu_info(self.h, ctypes.byref(fr), ctypes.byref(lv), ctypes.byref(fl),
                                                    ctypes.byref(fb), ctypes.byref(pp)))
        return {"fronts": fr.value, "levels": lv.value, "flops": fl.value, "factor_bytes": fb.value,
                "perturbed_pivots": pp.value}

    def close(self):
        if getattr(self, "h", None):
            self.ctx.L.fq_sparse_lu_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _krylov(fn: str, a: Matrix, b_ptr: int, x_ptr: int, inv_diag_ptr: int = 0, opts=None) -> Report:
    rep = _Report()
    opts = opts or SolveOpts.default()
    L = a.ctx.L
    s = getattr(L, fn)(a.ctx.h, a.h, _P(inv_diag_ptr) if inv_diag_ptr else None, _P(b_ptr), _P(x_ptr),
                       ctypes.byref(opts), ctypes.byref(rep))
    if s not in (0, 3):
        a.ctx.check(s, fn)
    return Report.of(rep)


def minres(a: Matrix, b_ptr: int, x_ptr: int, inv_diag_ptr: int = 0, opts=None) -> Report:
    """krylov::minres on device pointers (FP64)."""
    return _krylov("fq_minres", a, b_ptr, x_ptr, inv_diag_ptr, opts)


def cg(a: Matrix, b_ptr: int, x_ptr: int, inv_diag_ptr: int = 0, opts=None) -> Report:
    """krylov::cg on device pointers (FP64)."""
    return _krylov("fq_cg", a, b_ptr, x_ptr, inv_diag_ptr, opts)


def hx_cg(mesh: Mesh, grade: int, bc: int, rhs: np.ndarray, opts: Optional[SolveOpts] = None):
    """GradeKHodgeHx::with_multigrid(..).solve (formoniq/src/hx.rs): HX-preconditioned CG on hdif_gram(grade)."""
    rhs = np.ascontiguousarray(rhs, np.float64)
    x = np.zeros_like(rhs)
    rep = _Report()
    opts = opts or SolveOpts.default()
    s = mesh.ctx.L.fq_hx_cg(mesh.ctx.h, mesh.h, int(grade), int(bc), _dp(rhs), _dp(x), ctypes.byref(opts),
                            ctypes.byref(rep))
    if s not in (0, 3):
        mesh.ctx.check(s, "fq_hx_cg")
    return x, Report.of(rep)


def hx_apply(mesh: Mesh, grade: int, bc: int, r: np.ndarray) -> np.ndarray:
    """One application y = B r of the grade-`grade` HX preconditioner (AuxiliarySpace::apply)."""
    r = np.ascontiguousarray(r, np.float64)
    y = np.zeros_like(r)
    mesh.ctx.check(mesh.ctx.L.fq_hx_apply(mesh.ctx.h, mesh.h, int(grade), int(bc), _dp(r), _dp(y)), "fq_hx_apply")
    return y


class Server:
    """The serving loop (fq_server_*): lanes with their own streams, HBM-budget
    admission, meshes and solver state resident between requests."""

    def __init__(self, device: int = 0, lanes: int = 4, budget_bytes: int = 0, cache: bool = True):
        self.L = load()
        h = _P()
        s = self.L.fq_server_create(int(device), int(lanes), int(budget_bytes), int(bool(cache)), ctypes.byref(h))
        if s != 0:
            raise FqError(s, f"fq_server_create: {_STATUS.get(s, s)}")
        self.h = h
        self._keep = {}

    def submit(self, kind: int, dim: int, nbox: int, grade: int = 0, bc: int = FQ_ABSOLUTE, minkowski: bool = False,
               jitter: float = 0.1, seed: int = 0, mass_term: float = 1.5, arrival_ms: float = -1.0,
               lengths: Optional[np.ndarray] = None, source: Optional[np.ndarray] = None,
               solution: Optional[np.ndarray] = None, opts: Optional[SolveOpts] = None) -> int:
        keep = []
        r = _Request()
        r.kind, r.dim, r.nbox, r.grade, r.bc = int(kind), int(dim), int(nbox), int(grade), int(bc)
        r.minkowski, r.jitter, r.seed, r.mass_term = int(bool(minkowski)), float(jitter), int(seed), float(mass_term)
        r.arrival_ms = float(arrival_ms)
        for name, arr in (("lengths", lengths), ("source", source), ("solution", solution)):
            if arr is not None:
                if arr.dtype != np.float64 or not arr.flags["C_CONTIGUOUS"]:
                    raise ValueError(f"{name} must be a contiguous float64 array")
                keep.append(arr)
                setattr(r, name, arr.ctypes.data)
        r.opts = opts or SolveOpts.default()
        t = ctypes.c_uint64()
        s = self.L.fq_server_submit(self.h, ctypes.byref(r), ctypes.byref(t))
        if s != 0:
            raise FqError(s, f"fq_server_submit: {_STATUS.get(s, s)}")
        self._keep[t.value] = keep
        return t.value

    def wait(self, ticket: int) -> dict:
        res = _Result()
        s = self.L.fq_server_wait(self.h, ctypes.c_uint64(ticket), ctypes.byref(res))
        if s != 0:
            raise FqError(s, f"fq_server_wait: {_STATUS.get(s, s)}")
        self._keep.pop(ticket, None)
        return {"status": res.status, "lane": res.lane, "report": Report.of(res.report), "queue_ms": res.queue_ms,
                "run_ms": res.run_ms, "latency_ms": res.latency_ms, "start_ms": res.start_ms, "end_ms": res.end_ms,
                "checksum": res.checksum, "ndofs": res.ndofs, "cache_hit": bool(res.cache_hit)}

    def stats(self) -> dict:
        st = _ServerStats()
        self.L.fq_server_get_stats(self.h, ctypes.byref(st))
        return {f: getattr(st, f) for f, _ in _ServerStats._fields_}

    def close(self):
        if self.h:
            self.L.fq_server_destroy(self.h)
            self.h = None
            self._keep.clear()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


class Batch:
    """Batched assembly of one form per mesh (fq_batch_*)."""

    def __init__(self, ctx: Context, meshes, grades, form: int = FQ_BATCH_HDIF):
        self.ctx, self.meshes, self.grades = ctx, list(meshes), [int(g) for g in grades]
        arr = (_P * len(self.meshes))(*[m.h for m in self.meshes])
        g = np.ascontiguousarray(self.grades, np.int32)
        h = _P()
        ctx.check(ctx.L.fq_batch_create(ctx.h, len(self.meshes), arr, g.ctypes.data_as(_I32P), int(form),
                                        ctypes.byref(h)), "fq_batch_create")
        self.h = h
        ctx._adopt(self)

    def tune(self, reps: int = 3):
        self.ctx.check(self.ctx.L.fq_batch_tune(self.h, int(reps)), "fq_batch_tune")

    def set_launch(self, element_grid: int = 0, scatter_tps: int = 1, scatter_grid: int = 0):
        self.ctx.check(self.ctx.L.fq_batch_set_launch(self.h, element_grid, scatter_tps, scatter_grid),
                       "fq_batch_set_launch")

    def set_element_launch(self, fused: bool, grid: int = 0):
        """The element pass as one fused launch over every class, or one per class
        (fq_batch_set_element_launch)."""
        self.ctx.check(self.ctx.L.fq_batch_set_element_launch(self.h, int(bool(fused)), int(grid)),
                       "fq_batch_set_element_launch")

    def fused_registers(self) -> int:
        return int(self.ctx.L.fq_batch_fused_registers())

    def assemble(self, check: bool = True):
        self.ctx.check(self.ctx.L.fq_batch_assemble(self.h, int(check)), "fq_batch_assemble")

    def assemble_per_mesh(self, check: bool = True):
        self.ctx.check(self.ctx.L.fq_batch_assemble_per_mesh(self.h, int(check)), "fq_batch_assemble_per_mesh")

    def info(self) -> dict:
        c, s = ctypes.c_int64(), ctypes.c_int64()
        k, n = ctypes.c_int(), ctypes.c_int()
        self.ctx.check(self.ctx.L.fq_batch_info(self.h, ctypes.byref(c), ctypes.byref(s), ctypes.byref(k),
                                                ctypes.byref(n)))
        tps, sg = ctypes.c_int(), ctypes.c_int()
        grids = (ctypes.c_int * 64)()
        self.ctx.L.fq_batch_launch_config(self.h, ctypes.byref(tps), ctypes.byref(sg), grids, 64)
        return {"cells": c.value, "slots": s.value, "classes": k.value, "launches_per_assembly": n.value,
                "scatter_threads_per_slot": tps.value, "scatter_grid": sg.value,
                "element_grids": list(grids)[:k.value]}

    def to_scipy(self, i: int):
        import scipy.sparse as sp

        nr, nnz = ctypes.c_int64(), ctypes.c_int64()
        self.ctx.check(self.ctx.L.fq_batch_matrix(self.h, int(i), ctypes.byref(nr), ctypes.byref(nnz), None, None,
                                                  None))
        rp = np.zeros(nr.value + 1, np.int32)
        ci = np.zeros(max(nnz.value, 1), np.int32)
        v = np.zeros(max(nnz.value, 1))
        self.ctx.check(self.ctx.L.fq_batch_copy_to_host(self.h, int(i), rp.ctypes.data_as(_I32P),
                                                        ci.ctypes.data_as(_I32P), _dp(v)))
        return sp.csr_matrix((v[:nnz.value], ci[:nnz.value], rp), shape=(nr.value, nr.value))

    def close(self):
        if self.h:
            self.ctx.L.fq_batch_destroy(self.h)
            self.h = None
