"""Python binding of the GB300 RSVD-Delta-t C ABI (include/rsvdt.h).

Mirrors the reference's hot-path interface (AliFarghadan/RSVD-Delta-t,
SourceCode/main.c:134-144): a Context holds the operator, the weights and
the working spectral block; `action`, `qr_all_freqs`, `svd_all_freqs`,
`power_iteration` and `run` stand in for DirectActionRK4 /
AdjointActionRK4, QRAllFreqs, SVDAllFreqs(BeforeAdjoint), PowerIterationRK4
and the main sequence. Errors raise RsvdtError carrying the library's status
code and message, as the reference's CHKERRQ/SETERRQ chain does.

There is no CPU fallback: the shared library must have been built
(`build.build_library`) and a CUDA device must be present.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

LIB_PATH = _build.LIB_PATH

OK, ERR_ARG, ERR_IO, ERR_OOM, ERR_CUDA, ERR_NOT_SPD, ERR_DIVERGED, ERR_TIMEOUT, ERR_STATE = range(9)
ADJOINT, DIRECT = 0, 1
PREC_C128, PREC_C64, PREC_C64_REFINE = 0, 1, 2
ENGINE_AUTO, ENGINE_STAGES, ENGINE_CLUSTER = 0, 1, 2
W_F_SQRT_INV, B, C_OUT, W_Q_SQRT, W_Q_SQRT_INV = range(5)

STATUS_NAMES = {0: "OK", 1: "ARG", 2: "IO", 3: "OOM", 4: "CUDA", 5: "NOT_SPD", 6: "DIVERGED",
                7: "TIMEOUT", 8: "STATE"}

# Every symbol include/rsvdt.h declares.
EXPORTED = [
    "rsvdt_default_params", "rsvdt_create", "rsvdt_destroy", "rsvdt_last_error",
    "rsvdt_set_operator", "rsvdt_set_operator_bcsr", "rsvdt_set_weight", "rsvdt_get_grid",
    "rsvdt_set_sketch", "rsvdt_random_sketch", "rsvdt_get_block", "rsvdt_action",
    "rsvdt_qr_all_freqs", "rsvdt_svd_all_freqs", "rsvdt_power_iteration", "rsvdt_set_checkpoint", "rsvdt_run",
    "rsvdt_debug_build",
    "rsvdt_get_results", "rsvdt_rk4_steps", "rsvdt_rk4_reset", "rsvdt_rk4_advance",
    "rsvdt_rk4_profile", "rsvdt_rk4_profile_ex", "rsvdt_set_forcing_block", "rsvdt_get_forcing_block",
    "rsvdt_synchronize", "rsvdt_stream", "rsvdt_launch_count",
    "rsvdt_qr_all_freqs_noalloc", "rsvdt_trans_grid", "rsvdt_trans_run",
    "rsvdt_set_capacity_mode", "rsvdt_get_capacity", "rsvdt_get_result_cols", "rsvdt_device_memory",
    "rsvdt_set_lanes_per_row", "rsvdt_get_lanes_per_row", "rsvdt_get_timings", "rsvdt_reset_timings",
    "rsvdt_set_step_engine", "rsvdt_get_step_engine",
    "rsvdt_batch_create", "rsvdt_batch_destroy", "rsvdt_batch_last_error", "rsvdt_batch_add",
    "rsvdt_batch_set_sketch", "rsvdt_batch_random_sketch", "rsvdt_batch_run", "rsvdt_batch_get_results",
    "rsvdt_batch_get_grid", "rsvdt_batch_get_tuning", "rsvdt_batch_values_per_lane", "rsvdt_batch_set_launch_shape",
    "rsvdt_batch_launch_count",
    "rsvdt_mlp_create", "rsvdt_mlp_destroy", "rsvdt_mlp_last_error", "rsvdt_mlp_param_count",
    "rsvdt_mlp_set_params", "rsvdt_mlp_get_params", "rsvdt_mlp_forward", "rsvdt_mlp_gradients",
    "rsvdt_mlp_train",
]


def qr_all_freqs_noalloc(Y_dev: int, Q_dev: int, rows: int, nw: int, k: int, stream) -> None:
    """Binding of rsvdt_qr_all_freqs_noalloc: orthonormalises each
    frequency block of a caller-allocated device array (device pointers as
    integers, layout [row][iw][k] complex128) without allocating any device
    memory. `stream` is a cudaStream_t as an integer (e.g. a torch stream's
    `cuda_stream`), or None / 0 for the legacy default stream, which
    synchronises with every blocking stream and so breaks a capture open on
    one of them. Raises RsvdtError with the library's message on failure."""
    lib = load_library()
    buf = C.create_string_buffer(512)
    st = lib.rsvdt_qr_all_freqs_noalloc(C.c_void_p(Y_dev), C.c_void_p(Q_dev), rows, nw, k,
                                        C.c_void_p(stream) if stream else None, buf, len(buf))
    if st != OK:
        raise RsvdtError(st, buf.value.decode())


class Params(C.Structure):
    _fields_ = [
        ("k", C.c_int64), ("q", C.c_int64), ("Nw", C.c_int64), ("w", C.c_double),
        ("TwoPI", C.c_int32), ("dt", C.c_double), ("TransientLength", C.c_double),
        ("TransientRemoval", C.c_int32), ("DiscFlg", C.c_int32), ("beta", C.c_double),
        ("precision", C.c_int32), ("Display", C.c_int32),
    ]


class Grid(C.Structure):
    _fields_ = [
        ("w", C.c_double), ("dt", C.c_double), ("Ns", C.c_int64), ("Nt", C.c_int64),
        ("ResRatio", C.c_int64), ("Nw_eff", C.c_int64), ("N", C.c_int64), ("Nb", C.c_int64),
        ("Nc", C.c_int64),
    ]


class TransParams(C.Structure):
    _fields_ = [
        ("periods", C.c_int64), ("save_mod", C.c_int64), ("div_val", C.c_double), ("con_val", C.c_double),
        ("save", C.c_int32), ("removal_est", C.c_int32),
    ]


class TransInfo(C.Structure):
    _fields_ = [
        ("dt", C.c_double), ("Nt_period", C.c_int64), ("rend", C.c_int64), ("n_saved", C.c_int64),
        ("steps", C.c_int64), ("stop", C.c_int32), ("last_norm", C.c_double),
    ]


TRANS_DONE, TRANS_NAN, TRANS_DIVERGED, TRANS_CONVERGED = range(4)
TRANS_SNAPSHOT_FN = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_int64, C.POINTER(C.c_double), C.c_int64)
TRANS_ESTIMATE_FN = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_int64, C.POINTER(C.c_double), C.POINTER(C.c_double),
                                C.c_int64)
CHECKPOINT_FN = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_int32, C.c_void_p)


class RsvdtError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"rsvdt error {STATUS_NAMES.get(status, status)}: {msg}")
        self.status = status


_lib = None


def load_library(path: str | None = None) -> C.CDLL:
    """Loads lib/librsvdt.so (or the file named by the RSVDT_LIBRARY
    environment variable, e.g. the debug build); raises if it has not been
    built."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or os.environ.get("RSVDT_LIBRARY") or LIB_PATH
    if not os.path.exists(path):
        raise RuntimeError(f"CUDA library {path} is missing: run build.build_library() first")
    lib = C.CDLL(path)
    P = C.POINTER
    vp = C.c_void_p
    d = P(C.c_double)
    i64 = C.c_int64
    sig = {
        "rsvdt_default_params": (None, [P(Params)]),
        "rsvdt_create": (C.c_int, [P(Params), P(vp)]),
        "rsvdt_destroy": (None, [vp]),
        "rsvdt_last_error": (C.c_char_p, [vp]),
        "rsvdt_set_operator": (C.c_int, [vp, i64, P(i64), P(i64), d]),
        "rsvdt_set_operator_bcsr": (C.c_int, [vp, i64, C.c_int32, P(i64), P(i64), d]),
        "rsvdt_set_weight": (C.c_int, [vp, C.c_int, i64, i64, P(i64), P(i64), d]),
        "rsvdt_get_grid": (C.c_int, [vp, P(Grid)]),
        "rsvdt_set_sketch": (C.c_int, [vp, d, i64, i64]),
        "rsvdt_random_sketch": (C.c_int, [vp, C.c_uint64]),
        "rsvdt_get_block": (C.c_int, [vp, d, i64, P(i64)]),
        "rsvdt_action": (C.c_int, [vp, C.c_int]),
        "rsvdt_qr_all_freqs": (C.c_int, [vp]),
        "rsvdt_svd_all_freqs": (C.c_int, [vp, C.c_int32]),
        "rsvdt_power_iteration": (C.c_int, [vp]),
        "rsvdt_set_checkpoint": (C.c_int, [vp, C.c_void_p, C.c_void_p]),
        "rsvdt_debug_build": (C.c_int32, []),
        "rsvdt_run": (C.c_int, [vp]),
        "rsvdt_get_results": (C.c_int, [vp, d, i64, d, i64, d]),
        "rsvdt_rk4_steps": (C.c_int, [vp, C.c_int, i64, i64, d, d]),
        "rsvdt_rk4_reset": (C.c_int, [vp, C.c_int]),
        "rsvdt_rk4_advance": (C.c_int, [vp, C.c_int, i64, i64]),
        "rsvdt_rk4_profile": (C.c_int, [vp, C.c_int, i64, i64, d]),
        "rsvdt_rk4_profile_ex": (C.c_int, [vp, C.c_int, i64, i64, d]),
        "rsvdt_set_forcing_block": (C.c_int, [vp, C.c_int32]),
        "rsvdt_get_forcing_block": (C.c_int32, [vp]),
        "rsvdt_qr_all_freqs_noalloc": (C.c_int, [vp, vp, i64, i64, i64, vp, C.c_char_p, i64]),
        "rsvdt_set_capacity_mode": (C.c_int, [vp, i64, C.c_int32]),
        "rsvdt_get_capacity": (C.c_int, [vp, P(i64)]),
        "rsvdt_device_memory": (C.c_int, [P(i64), P(i64)]),
        "rsvdt_get_timings": (C.c_int, [vp, C.c_char_p, i64]),
        "rsvdt_reset_timings": (C.c_int, [vp]),
        "rsvdt_set_lanes_per_row": (C.c_int, [vp, C.c_int32]),
        "rsvdt_get_lanes_per_row": (C.c_int32, [vp]),
        "rsvdt_set_step_engine": (C.c_int, [vp, C.c_int32]),
        "rsvdt_get_step_engine": (C.c_int32, [vp]),
        "rsvdt_get_result_cols": (C.c_int, [vp, P(i64), i64, d, i64, d, i64]),
        "rsvdt_trans_grid": (C.c_int, [vp, P(TransParams), P(TransInfo)]),
        "rsvdt_trans_run": (C.c_int, [vp, P(TransParams), d, d, TRANS_SNAPSHOT_FN, TRANS_ESTIMATE_FN, vp,
                                      P(TransInfo)]),
        "rsvdt_batch_create": (C.c_int, [C.c_int32, P(vp)]),
        "rsvdt_batch_destroy": (None, [vp]),
        "rsvdt_batch_last_error": (C.c_char_p, [vp]),
        "rsvdt_batch_add": (C.c_int, [vp, P(Params), i64, P(i64), P(i64), d, P(C.c_int32)]),
        "rsvdt_batch_set_sketch": (C.c_int, [vp, C.c_int32, d, i64, i64]),
        "rsvdt_batch_random_sketch": (C.c_int, [vp, C.c_int32, C.c_uint64]),
        "rsvdt_batch_run": (C.c_int, [vp]),
        "rsvdt_batch_get_results": (C.c_int, [vp, C.c_int32, d, i64, d, i64, d]),
        "rsvdt_batch_get_grid": (C.c_int, [vp, C.c_int32, P(Grid)]),
        "rsvdt_batch_get_tuning": (C.c_int, [vp, P(C.c_int32), P(C.c_int32), d]),
        "rsvdt_batch_values_per_lane": (C.c_int32, [vp]),
        "rsvdt_batch_set_launch_shape": (C.c_int, [vp, C.c_int32, C.c_int32, C.c_int32]),
        "rsvdt_batch_launch_count": (i64, [vp]),
        "rsvdt_mlp_create": (C.c_int, [C.c_int32, P(C.c_int32), C.c_uint64, P(vp)]),
        "rsvdt_mlp_destroy": (None, [vp]),
        "rsvdt_mlp_last_error": (C.c_char_p, [vp]),
        "rsvdt_mlp_param_count": (i64, [vp]),
        "rsvdt_mlp_set_params": (C.c_int, [vp, P(C.c_float)]),
        "rsvdt_mlp_get_params": (C.c_int, [vp, P(C.c_float)]),
        "rsvdt_mlp_forward": (C.c_int, [vp, P(C.c_float), i64, P(C.c_float)]),
        "rsvdt_mlp_gradients": (C.c_int, [vp, P(C.c_float), P(C.c_float), i64, P(C.c_float), P(C.c_float)]),
        "rsvdt_mlp_train": (C.c_int, [vp, P(C.c_float), P(C.c_float), i64, i64, i64, C.c_float, C.c_uint64,
                                      P(C.c_float)]),
        "rsvdt_synchronize": (C.c_int, [vp]),
        "rsvdt_stream": (vp, [vp]),
        "rsvdt_launch_count": (i64, [vp]),
    }
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


def default_params(**kw) -> Params:
    lib = load_library()
    p = Params()
    lib.rsvdt_default_params(C.byref(p))
    for k, v in kw.items():
        if not hasattr(p, k):
            raise KeyError(k)
        setattr(p, k, v)
    return p


def _dptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _iptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_int64))


def _csr_arrays(indptr, indices, data):
    rp = np.ascontiguousarray(indptr, dtype=np.int64)
    ci = np.ascontiguousarray(indices, dtype=np.int64)
    va = np.ascontiguousarray(data, dtype=np.complex128)
    return rp, ci, va


class Context:
    """One resolvent problem on the GPU (one CUDA stream, device-resident
    operator, weights and spectral blocks)."""

    def __init__(self, params: Params | None = None, **kw):
        self._lib = load_library()
        self._h = C.c_void_p()
        p = params if params is not None else default_params(**kw)
        self.params = p
        st = self._lib.rsvdt_create(C.byref(p), C.byref(self._h))
        if st != OK:
            msg = self._lib.rsvdt_last_error(self._h).decode() if self._h else "create failed"
            self.close()
            raise RsvdtError(st, msg)

    def close(self):
        if getattr(self, "_h", None):
            self._lib.rsvdt_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _check(self, st: int):
        if st != OK:
            raise RsvdtError(st, self._lib.rsvdt_last_error(self._h).decode())

    # -------------------------------------------------------- set-up
    def set_operator(self, A) -> None:
        """A: scipy.sparse matrix (converted to CSR) or (indptr, indices, data)."""
        if hasattr(A, "tocsr"):
            A = A.tocsr()
            A.sort_indices()
            n = A.shape[0]
            rp, ci, va = _csr_arrays(A.indptr, A.indices, A.data)
        else:
            rp, ci, va = _csr_arrays(*A)
            n = rp.size - 1
        self._check(self._lib.rsvdt_set_operator(self._h, n, _iptr(rp), _iptr(ci), _dptr(va.view(np.float64))))

    def set_operator_bcsr(self, browptr, bcol, blocks) -> None:
        """blocks: (nblocks, bs, bs) complex array, row-major inside a block."""
        rp = np.ascontiguousarray(browptr, dtype=np.int64)
        bc = np.ascontiguousarray(bcol, dtype=np.int64)
        bl = np.ascontiguousarray(blocks, dtype=np.complex128)
        bs = bl.shape[1]
        self._check(self._lib.rsvdt_set_operator_bcsr(self._h, rp.size - 1, bs, _iptr(rp), _iptr(bc),
                                                      _dptr(bl.view(np.float64))))

    def set_weight(self, which: int, M) -> None:
        M = M.tocsr()
        M.sort_indices()
        rp, ci, va = _csr_arrays(M.indptr, M.indices, M.data)
        self._check(self._lib.rsvdt_set_weight(self._h, which, M.shape[0], M.shape[1], _iptr(rp), _iptr(ci),
                                               _dptr(va.view(np.float64))))

    def grid(self) -> Grid:
        g = Grid()
        self._check(self._lib.rsvdt_get_grid(self._h, C.byref(g)))
        return g

    def set_sketch(self, F: np.ndarray) -> None:
        """F: Nb x (k*Nw_eff) complex, frequency-major columns (iw*k + ik)."""
        F = np.asfortranarray(F, dtype=np.complex128)
        self._check(self._lib.rsvdt_set_sketch(self._h, F.ctypes.data_as(C.POINTER(C.c_double)), F.shape[0],
                                               F.shape[1]))
        self._k = F.shape[1] // self.grid().Nw_eff

    def random_sketch(self, seed: int) -> None:
        self._check(self._lib.rsvdt_random_sketch(self._h, seed))

    # -------------------------------------------------------- algorithm
    def action(self, direction: int) -> None:
        self._check(self._lib.rsvdt_action(self._h, direction))

    def qr_all_freqs(self) -> None:
        self._check(self._lib.rsvdt_qr_all_freqs(self._h))

    def svd_all_freqs(self, before_adjoint: bool) -> None:
        self._check(self._lib.rsvdt_svd_all_freqs(self._h, 1 if before_adjoint else 0))

    def power_iteration(self) -> None:
        self._check(self._lib.rsvdt_power_iteration(self._h))

    def set_checkpoint(self, fn) -> None:
        """fn(sweep) is called after the second QR of every power sweep
        (rsvdt_set_checkpoint); it may read the block with get_block(). A
        true return value stops the run (RsvdtError, ERR_STATE). None
        removes the hook."""
        if fn is None:
            self._ckpt = None
            self._check(self._lib.rsvdt_set_checkpoint(self._h, None, None))
            return

        def tramp(user, sweep, ctx):
            try:
                return 1 if fn(int(sweep)) else 0
            except Exception:
                return 1

        self._ckpt = CHECKPOINT_FN(tramp)
        self._check(self._lib.rsvdt_set_checkpoint(self._h, C.cast(self._ckpt, C.c_void_p), None))

    def run(self) -> None:
        self._check(self._lib.rsvdt_run(self._h))

    # -------------------------------------------------------- read back
    def get_block(self) -> np.ndarray:
        rows = C.c_int64()
        self._check(self._lib.rsvdt_get_block(self._h, None, 1, C.byref(rows)))
        g = self.grid()
        k = self.k
        out = np.zeros((rows.value, k * g.Nw_eff), dtype=np.complex128, order="F")
        self._check(self._lib.rsvdt_get_block(self._h, out.ctypes.data_as(C.POINTER(C.c_double)), rows.value,
                                              C.byref(rows)))
        return out

    @property
    def k(self) -> int:
        return int(self._k) if hasattr(self, "_k") else int(self.params.k)

    def get_results(self, U: bool = True, V: bool = True):
        """(U, V, S); U or V is None when not requested."""
        g = self.grid()
        ncol = self.k * g.Nw_eff
        dp = C.POINTER(C.c_double)
        Uo = np.zeros((g.Nc, ncol), dtype=np.complex128, order="F") if U else None
        Vo = np.zeros((g.Nb, ncol), dtype=np.complex128, order="F") if V else None
        S = np.zeros((self.k, g.Nw_eff), dtype=np.float64, order="F")
        self._check(self._lib.rsvdt_get_results(self._h, Uo.ctypes.data_as(dp) if U else None, g.Nc,
                                                Vo.ctypes.data_as(dp) if V else None, g.Nb, S.ctypes.data_as(dp)))
        return Uo, Vo, S

    def rk4_steps(self, direction: int, i0: int, nsteps: int, y: np.ndarray, F3: np.ndarray):
        """Advances the host state y, F3 (N x k complex, Fortran order) in place."""
        y = np.asfortranarray(y, dtype=np.complex128)
        F3 = np.asfortranarray(F3, dtype=np.complex128)
        self._check(self._lib.rsvdt_rk4_steps(self._h, direction, i0, nsteps,
                                              y.ctypes.data_as(C.POINTER(C.c_double)),
                                              F3.ctypes.data_as(C.POINTER(C.c_double))))
        return y, F3

    def rk4_reset(self, direction: int) -> None:
        self._check(self._lib.rsvdt_rk4_reset(self._h, direction))

    def rk4_advance(self, direction: int, i0: int, nsteps: int) -> None:
        self._check(self._lib.rsvdt_rk4_advance(self._h, direction, i0, nsteps))

    def rk4_profile(self, direction: int, i0: int, nsteps: int) -> list:
        """Per-stage device time (ms, summed over nsteps) from CUDA events."""
        out = np.zeros(4)
        self._check(self._lib.rsvdt_rk4_profile(self._h, direction, i0, nsteps,
                                                out.ctypes.data_as(C.POINTER(C.c_double))))
        return out.tolist()

    def rk4_profile_ex(self, direction: int, i0: int, nsteps: int) -> list:
        """[stage 1, 2, 3, 4, forcing block] device time (ms, summed over
        nsteps) from CUDA events (rsvdt_rk4_profile_ex)."""
        out = np.zeros(5)
        self._check(self._lib.rsvdt_rk4_profile_ex(self._h, direction, i0, nsteps,
                                                   out.ctypes.data_as(C.POINTER(C.c_double))))
        return out.tolist()

    def set_forcing_block(self, steps: int) -> None:
        """Forcing synthesised ahead in blocks of `steps` steps (complex64
        block-row stages; 0 = in stage 1, -1 = automatic)."""
        self._check(self._lib.rsvdt_set_forcing_block(self._h, steps))

    def forcing_block(self) -> int:
        return int(self._lib.rsvdt_get_forcing_block(self._h))

    def timings(self) -> dict:
        """Wall time per phase (rsvdt_get_timings) as a dict."""
        import json

        buf = C.create_string_buffer(1024)
        self._check(self._lib.rsvdt_get_timings(self._h, buf, len(buf)))
        return json.loads(buf.value.decode())

    def reset_timings(self) -> None:
        self._check(self._lib.rsvdt_reset_timings(self._h))

    def set_lanes_per_row(self, lanes: int) -> None:
        """1: stage kernels with one thread per row; 2/4/8: the batched
        stage kernel with that many lanes per row; 0: automatic."""
        self._check(self._lib.rsvdt_set_lanes_per_row(self._h, lanes))

    def lanes_per_row(self) -> int:
        return int(self._lib.rsvdt_get_lanes_per_row(self._h))

    def set_step_engine(self, engine: int) -> None:
        """ENGINE_AUTO, ENGINE_STAGES or ENGINE_CLUSTER (rsvdt_set_step_engine)."""
        self._check(self._lib.rsvdt_set_step_engine(self._h, engine))

    def step_engine(self) -> int:
        """The engine the next stepping uses (STAGES or CLUSTER)."""
        return int(self._lib.rsvdt_get_step_engine(self._h))

    # -------------------------------------------------------- capacity mode
    def set_capacity_mode(self, kc: int = 0, u_c64: bool = False) -> None:
        """Chunked actions, in-place blocks, U in host memory (call before
        set_operator for problems whose resident buffers would not fit)."""
        self._check(self._lib.rsvdt_set_capacity_mode(self._h, kc, 1 if u_c64 else 0))

    def capacity_chunk(self) -> int:
        kc = C.c_int64()
        self._check(self._lib.rsvdt_get_capacity(self._h, C.byref(kc)))
        return kc.value

    def get_result_cols(self, cols, U: bool = True, V: bool = True):
        """Columns (iw*k + ik) of U and V after run()."""
        g = self.grid()
        cols = np.ascontiguousarray(cols, dtype=np.int64)
        Uo = np.zeros((g.Nc, cols.size), dtype=np.complex128, order="F") if U else None
        Vo = np.zeros((g.Nb, cols.size), dtype=np.complex128, order="F") if V else None
        dp = C.POINTER(C.c_double)
        self._check(self._lib.rsvdt_get_result_cols(
            self._h, _iptr(cols), cols.size, Uo.ctypes.data_as(dp) if U else None, g.Nc,
            Vo.ctypes.data_as(dp) if V else None, g.Nb))
        return Uo, Vo

    # -------------------------------------------------------- transient run
    @staticmethod
    def _trans_params(periods=1, save_mod=100, div_val=1e3, con_val=1e-8, save=False, removal_est=False):
        # Defaults of SourceCode/ReadUserInput.c:142-171.
        return TransParams(int(periods), int(save_mod), float(div_val), float(con_val), int(bool(save)),
                           int(bool(removal_est)))

    def trans_grid(self, **kw) -> TransInfo:
        info = TransInfo()
        tp = self._trans_params(**kw)
        self._check(self._lib.rsvdt_trans_grid(self._h, C.byref(tp), C.byref(info)))
        return info

    def trans_run(self, q0: np.ndarray, **kw):
        """Transient simulation from q0 (N complex). Returns (q_last, norms,
        info, snapshots {pos: q}, estimates [(period, initial, updated)]);
        snapshots are kept only with save=True."""
        tp = self._trans_params(**kw)
        info = TransInfo()
        self._check(self._lib.rsvdt_trans_grid(self._h, C.byref(tp), C.byref(info)))
        q = np.ascontiguousarray(q0, dtype=np.complex128).copy()
        norms = np.zeros(info.n_saved)
        snaps, ests = {}, []

        def on_snap(_u, pos, ptr, n):
            snaps[int(pos)] = np.ctypeslib.as_array(ptr, shape=(2 * n,)).view(np.complex128).copy()
            return 0

        def on_est(_u, period, pi, pu, count):
            ests.append((int(period), np.ctypeslib.as_array(pi, shape=(count,)).copy(),
                         np.ctypeslib.as_array(pu, shape=(count,)).copy()))
            return 0

        fs, fe = TRANS_SNAPSHOT_FN(on_snap), TRANS_ESTIMATE_FN(on_est)
        self._check(self._lib.rsvdt_trans_run(self._h, C.byref(tp), _dptr(q.view(np.float64)), _dptr(norms), fs, fe,
                                              None, C.byref(info)))
        return q, norms, info, snaps, ests

    def synchronize(self) -> None:
        self._check(self._lib.rsvdt_synchronize(self._h))

    def stream(self) -> int:
        return int(self._lib.rsvdt_stream(self._h) or 0)

    def launch_count(self) -> int:
        return int(self._lib.rsvdt_launch_count(self._h))


class Batch:
    """Many independent problems solved together (rsvdt_batch_*): every
    action runs for all problems at once with lockstep batched RK4 stages."""

    def __init__(self, precision: int = PREC_C128):
        self._lib = load_library()
        self._h = C.c_void_p()
        self._k = []
        st = self._lib.rsvdt_batch_create(precision, C.byref(self._h))
        if st != OK:
            msg = self._lib.rsvdt_batch_last_error(self._h).decode() if self._h else "batch creation failed"
            self.close()
            raise RsvdtError(st, msg)

    def close(self):
        if getattr(self, "_h", None):
            self._lib.rsvdt_batch_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, st: int):
        if st != OK:
            raise RsvdtError(st, self._lib.rsvdt_batch_last_error(self._h).decode())

    def add(self, params: Params, A) -> int:
        A = A.tocsr()
        A.sort_indices()
        rp, ci, va = _csr_arrays(A.indptr, A.indices, A.data)
        idx = C.c_int32()
        self._check(self._lib.rsvdt_batch_add(self._h, C.byref(params), A.shape[0], _iptr(rp), _iptr(ci),
                                              _dptr(va.view(np.float64)), C.byref(idx)))
        self._k.append(int(params.k))
        return idx.value

    def grid(self, index: int) -> Grid:
        g = Grid()
        self._check(self._lib.rsvdt_batch_get_grid(self._h, index, C.byref(g)))
        return g

    def set_sketch(self, index: int, F: np.ndarray) -> None:
        F = np.asfortranarray(F, dtype=np.complex128)
        self._check(self._lib.rsvdt_batch_set_sketch(self._h, index, F.ctypes.data_as(C.POINTER(C.c_double)),
                                                     F.shape[0], F.shape[1]))
        self._k[index] = F.shape[1] // self.grid(index).Nw_eff

    def random_sketch(self, index: int, seed: int) -> None:
        self._check(self._lib.rsvdt_batch_random_sketch(self._h, index, seed))

    def run(self) -> None:
        self._check(self._lib.rsvdt_batch_run(self._h))

    def get_results(self, index: int):
        g = self.grid(index)
        k = self._k[index]
        ncol = k * g.Nw_eff
        U = np.zeros((g.Nc, ncol), dtype=np.complex128, order="F")
        V = np.zeros((g.Nb, ncol), dtype=np.complex128, order="F")
        S = np.zeros((k, g.Nw_eff), dtype=np.float64, order="F")
        self._check(self._lib.rsvdt_batch_get_results(self._h, index, U.ctypes.data_as(C.POINTER(C.c_double)), g.Nc,
                                                      V.ctypes.data_as(C.POINTER(C.c_double)), g.Nb,
                                                      S.ctypes.data_as(C.POINTER(C.c_double))))
        return U, V, S

    def tuning(self):
        th, fs, ms = C.c_int32(), C.c_int32(), C.c_double()
        self._check(self._lib.rsvdt_batch_get_tuning(self._h, C.byref(th), C.byref(fs), C.byref(ms)))
        return th.value, fs.value, ms.value

    def values_per_lane(self) -> int:
        return int(self._lib.rsvdt_batch_values_per_lane(self._h))

    def set_launch_shape(self, threads: int, lanes_per_row: int = 1, values_per_lane: int = 1) -> None:
        """Fixes the launch shape (threads = 0: autotune again)."""
        self._check(self._lib.rsvdt_batch_set_launch_shape(self._h, threads, lanes_per_row, values_per_lane))

    def launch_count(self) -> int:
        return int(self._lib.rsvdt_batch_launch_count(self._h))


def _fptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_float))


class Mlp:
    """The learned sketch's network (rsvdt_mlp_*): GELU MLP with bf16
    weights and FP32 accumulation, trained on the GPU."""

    def __init__(self, widths, seed: int = 0):
        self._lib = load_library()
        self._h = C.c_void_p()
        self.widths = [int(x) for x in widths]
        w = (C.c_int32 * len(self.widths))(*self.widths)
        st = self._lib.rsvdt_mlp_create(len(self.widths) - 1, w, seed, C.byref(self._h))
        if st != OK:
            msg = self._lib.rsvdt_mlp_last_error(self._h).decode() if self._h else "network creation failed"
            self.close()
            raise RsvdtError(st, msg)

    def close(self):
        if getattr(self, "_h", None):
            self._lib.rsvdt_mlp_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, st):
        if st != OK:
            raise RsvdtError(st, self._lib.rsvdt_mlp_last_error(self._h).decode())

    @property
    def n_params(self) -> int:
        return int(self._lib.rsvdt_mlp_param_count(self._h))

    def get_params(self) -> np.ndarray:
        p = np.zeros(self.n_params, dtype=np.float32)
        self._check(self._lib.rsvdt_mlp_get_params(self._h, _fptr(p)))
        return p

    def set_params(self, p: np.ndarray) -> None:
        p = np.ascontiguousarray(p, dtype=np.float32)
        self._check(self._lib.rsvdt_mlp_set_params(self._h, _fptr(p)))

    def forward(self, X: np.ndarray) -> np.ndarray:
        X = np.ascontiguousarray(X, dtype=np.float32)
        Y = np.zeros((X.shape[0], self.widths[-1]), dtype=np.float32)
        self._check(self._lib.rsvdt_mlp_forward(self._h, _fptr(X), X.shape[0], _fptr(Y)))
        return Y

    def gradients(self, X: np.ndarray, T: np.ndarray):
        X = np.ascontiguousarray(X, dtype=np.float32)
        T = np.ascontiguousarray(T, dtype=np.float32)
        g = np.zeros(self.n_params, dtype=np.float32)
        loss = C.c_float()
        self._check(self._lib.rsvdt_mlp_gradients(self._h, _fptr(X), _fptr(T), X.shape[0], C.byref(loss), _fptr(g)))
        return float(loss.value), g

    def train(self, X: np.ndarray, T: np.ndarray, batch: int, steps: int, lr: float, seed: int = 0) -> float:
        X = np.ascontiguousarray(X, dtype=np.float32)
        T = np.ascontiguousarray(T, dtype=np.float32)
        loss = C.c_float()
        self._check(self._lib.rsvdt_mlp_train(self._h, _fptr(X), _fptr(T), X.shape[0], batch, steps, lr, seed,
                                              C.byref(loss)))
        return float(loss.value)
