"""Python mirror of the three stage programs over the kevd C ABI.

Stage functions keep the reference programs' vocabulary and error behaviour:

* ``calibrate`` / ``select_bandwidth`` -- ``./cuband`` (ks_bandwidth.cu), the
  pair-sum sweep and the slope/arg-max selection written to ``bw0.out``;
* ``rpcholesky`` -- ``./cuarpclm`` (ks_arpclm.cu), pivots in acceptance order
  (``/spiv``), the per-round table and ``linv`` (``/linv``);
* ``bistochastic_evd`` -- ``./cukevd`` (ks_kevd.cu), eigenvalues ascending
  (``/lam``) and the N x k_out eigenvector block ``/U``; the reference's abort
  codes become ``KevdError`` with the matching status.

Device memory is held in torch tensors (plumbing only); every compute call is
a CUDA kernel of libkevd.so.  Nothing here falls back to a CPU path.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np
import torch

from . import _lib
from ._lib import (KEVD_FP64, KEVD_MIXED, EvdDump, EvdInfo, KevdError, RpcholParams, RpcholResult,
                   check)

PRECISIONS = {"fp64": KEVD_FP64, "mixed": KEVD_MIXED}


def _prec(p) -> int:
    if isinstance(p, str):
        return PRECISIONS[p]
    return int(p)


def _ptr(t: torch.Tensor | None):
    return C.c_void_p(t.data_ptr()) if t is not None else C.c_void_p(0)


def _np_ptr(a: np.ndarray | None):
    return C.c_void_p(a.ctypes.data) if a is not None else C.c_void_p(0)


def _stream():
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def _need_cuda(t: torch.Tensor, dtype, name: str):
    if not (isinstance(t, torch.Tensor) and t.is_cuda and t.dtype == dtype and t.is_contiguous()):
        raise ValueError(f"{name} must be a contiguous CUDA tensor of {dtype}")


class Context:
    """One kevd context (cuBLAS / cuSOLVER handles and device workspace)."""

    def __init__(self, device: int = 0):
        self.lib = _lib.load()
        self.device = device
        h = C.c_void_p()
        st = self.lib.kevd_ctx_create(device, C.byref(h))
        if st != 0:
            raise KevdError(st, "kevd_ctx_create failed")
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.lib.kevd_ctx_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, st):
        check(st, self.h)


# ---- views -----------------------------------------------------------------
def hankel_rows(ctx: Context, u: torch.Tensor, Ndata: int, M: int, Nq: int) -> torch.Tensor:
    _need_cuda(u, torch.float32, "u")
    N = Ndata - Nq + 1
    X = torch.empty((N * M, Nq), dtype=torch.float32, device=u.device)
    ctx._check(ctx.lib.kevd_hankel_rows(ctx.h, _ptr(u), Ndata, M, Nq, _ptr(X), _stream()))
    return X


def kernel_block(ctx: Context, X: torch.Tensor, scale: float, cols: torch.Tensor, rows=None,
                 row0: int = 0, nrows: int | None = None, precision="fp64") -> torch.Tensor:
    _need_cuda(X, torch.float32, "X")
    N, d = X.shape
    p = _prec(precision)
    if rows is not None:
        nrows = rows.numel()
    elif nrows is None:
        nrows = N - row0
    dt = torch.float64 if p == KEVD_FP64 else torch.float32
    out = torch.empty((nrows, cols.numel()), dtype=dt, device=X.device)
    ctx._check(ctx.lib.kevd_kernel_block(ctx.h, _ptr(X), N, d, float(scale), _ptr(rows), row0, nrows,
                                         _ptr(cols), cols.numel(), p, _ptr(out), cols.numel(), _stream()))
    return out


# ---- stage 1 ---------------------------------------------------------------
def calibrate(ctx: Context, X: torch.Tensor, scales, precision="mixed") -> np.ndarray:
    """sums[j] = sum_{i>l} exp(-scales[j] ||x_i - x_l||^2) (FP64, host).

    ``precision="mixed"``: the fused FP32-distance / exp2 pass;
    ``"fp64"``: its plain FP64 form (FP64 distances and exp)."""
    _need_cuda(X, torch.float32, "X")
    scales = np.ascontiguousarray(scales, dtype=np.float64)
    sums = np.zeros(scales.size, dtype=np.float64)
    N, d = X.shape
    fn = ctx.lib.kevd_calibrate_fp64 if _prec(precision) == KEVD_FP64 else ctx.lib.kevd_calibrate
    ctx._check(fn(ctx.h, _ptr(X), N, d, _np_ptr(scales), scales.size, _np_ptr(sums), _stream()))
    return sums


def calibrate_batched(ctx: Context, Xs, scales_list, tiles_per_item: int = 0) -> list:
    """calibrate() for many datasets (uneven N, d <= 128, <= 64 scales each) in
    one persistent launch over a device work queue of pair-tile ranges."""
    n = len(Xs)
    jobs = (_lib.CalibJob * n)()
    keep = []
    outs = []
    for q, (X, sc) in enumerate(zip(Xs, scales_list)):
        _need_cuda(X, torch.float32, "X")
        sc = np.ascontiguousarray(sc, dtype=np.float64)
        out = np.zeros(sc.size, dtype=np.float64)
        keep += [sc, out]
        outs.append(out)
        jobs[q] = _lib.CalibJob(X.data_ptr(), X.shape[0], X.shape[1], sc.size, sc.ctypes.data, out.ctypes.data)
    ctx._check(ctx.lib.kevd_calibrate_batched(ctx.h, jobs, n, int(tiles_per_item), _stream()))
    return outs


def calibrate_noalloc(X: torch.Tensor, scales) -> np.ndarray:
    """calibrate() without a context or any device allocation (fixed device
    scratch; at most 64 scales; concurrent calls on one GPU race)."""
    _need_cuda(X, torch.float32, "X")
    scales = np.ascontiguousarray(scales, dtype=np.float64)
    sums = np.zeros(scales.size, dtype=np.float64)
    N, d = X.shape
    check(_lib.load().kevd_calibrate_noalloc(_ptr(X), N, d, _np_ptr(scales), scales.size, _np_ptr(sums),
                                             _stream()))
    return sums


def select_bandwidth(bw, sums, NM: int) -> dict:
    """ks_bandwidth.cu:612-642: logS, centred slope, first arg-max, eopt, mdim."""
    lib = _lib.load()
    bw = np.ascontiguousarray(bw, dtype=np.float64)
    sums = np.ascontiguousarray(sums, dtype=np.float64)
    n = bw.size
    logS = np.zeros(n)
    slope = np.zeros(max(n - 2, 1))
    idmax = C.c_int32()
    eopt = C.c_double()
    mdim = C.c_double()
    st = lib.kevd_calibrate_select(_np_ptr(bw), _np_ptr(sums), n, NM, _np_ptr(logS), _np_ptr(slope),
                                   C.byref(idmax), C.byref(eopt), C.byref(mdim))
    check(st)
    return dict(logS=logS, slope=slope[: n - 2], idmax=idmax.value, eopt=eopt.value, mdim=mdim.value)


def bw0_text(bw, sel: dict) -> str:
    """bw0.out contents (ks_bandwidth.cu:645-655)."""
    logS, slope = sel["logS"], sel["slope"]
    lines = [f"{bw[i]:.5e} {logS[i]:.5e} {slope[i - 1]:.5e}" for i in range(1, len(bw) - 1)]
    return "\n".join(lines) + f"\n\n{sel['eopt']:.5e}\n{sel['mdim']:.5e}\n"


def pair_median(ctx: Context, X: torch.Tensor, pairs=None) -> float:
    """Lower median of ||x_i - x_l||^2 over all pairs i > l, or over given pairs."""
    _need_cuda(X, torch.float32, "X")
    N, d = X.shape
    out = C.c_double()
    if pairs is None:
        st = ctx.lib.kevd_pair_median(ctx.h, _ptr(X), N, d, None, None, 0, C.byref(out), _stream())
    else:
        pi, pl = pairs
        st = ctx.lib.kevd_pair_median(ctx.h, _ptr(X), N, d, _ptr(pi), _ptr(pl), pi.numel(), C.byref(out),
                                      _stream())
    ctx._check(st)
    return out.value


def log_sweep(median: float, n: int, lo: float = -10.0, hi: float = 10.0) -> np.ndarray:
    return float(median) * 2.0 ** np.linspace(lo, hi, n)


# ---- stage 2 ---------------------------------------------------------------
@dataclass
class Factorization:
    F: torch.Tensor          # N x ldF (columns [0, rank) valid)
    piv: np.ndarray          # rank pivots, acceptance order
    err: np.ndarray          # per-round trace error
    accepted: np.ndarray     # per-round accepted count
    rank: int
    rounds: int
    trace_error: float
    precision: int
    scale: float = 0.0

    @property
    def factor(self) -> torch.Tensor:
        return self.F[:, : self.rank]


def rpcholesky(ctx: Context, X: torch.Tensor, scale: float, k_max: int, block: int = 64,
               max_rounds: int | None = None, tol: float = 1e-10, err_target: float = 0.0,
               seed: int = 1234, uniforms: np.ndarray | None = None, precision="mixed",
               F: torch.Tensor | None = None) -> Factorization:
    _need_cuda(X, torch.float32, "X")
    N, d = X.shape
    p = _prec(precision)
    if max_rounds is None:
        max_rounds = max(1, 4 * ((k_max + block - 1) // block) + 8)
    dt = torch.float64 if p == KEVD_FP64 else torch.float32
    if F is None:
        F = torch.empty((N, k_max), dtype=dt, device=X.device)
    prm = RpcholParams()
    prm.k_max, prm.block, prm.max_rounds = k_max, block, max_rounds
    prm.tol, prm.err_target, prm.seed, prm.precision = tol, err_target, seed & (2**64 - 1), p
    u = None
    if uniforms is not None:
        u = np.ascontiguousarray(uniforms, dtype=np.float64)
        if u.size < max_rounds * 2 * block:
            raise ValueError("uniforms must hold max_rounds x 2 x block draws")
        prm.uniforms = u.ctypes.data_as(C.POINTER(C.c_double))
    piv = np.zeros(k_max, dtype=np.int64)
    err = np.zeros(max_rounds, dtype=np.float64)
    acc = np.zeros(max_rounds, dtype=np.int32)
    res = RpcholResult()
    ctx._check(ctx.lib.kevd_rpchol(ctx.h, _ptr(X), N, d, float(scale), C.byref(prm), _ptr(F), F.shape[1],
                                   _np_ptr(piv), _np_ptr(err), _np_ptr(acc), C.byref(res), _stream()))
    return Factorization(F=F, piv=piv[: res.rank].copy(), err=err[: res.rounds].copy(),
                         accepted=acc[: res.rounds].copy(), rank=res.rank, rounds=res.rounds,
                         trace_error=res.trace_error, precision=p, scale=float(scale))


def linv(ctx: Context, fac: Factorization) -> np.ndarray:
    """The reference's /linv: L^{-1} (r x r, lower) with L = F(S, :)."""
    r = fac.rank
    out = np.zeros((r, r), dtype=np.float64, order="F")
    piv = np.ascontiguousarray(fac.piv, dtype=np.int64)
    ctx._check(ctx.lib.kevd_linv_from_factor(ctx.h, _ptr(fac.F), fac.precision, fac.F.shape[1],
                                             _np_ptr(piv), r, out.ctypes.data, _stream()))
    return out


def factor_from_linv(ctx: Context, X: torch.Tensor, scale: float, piv, Linv: np.ndarray,
                     precision="fp64") -> torch.Tensor:
    """F = K(:, S) L^{-T} from the reference's stage-2 outputs."""
    _need_cuda(X, torch.float32, "X")
    N, d = X.shape
    p = _prec(precision)
    piv = np.ascontiguousarray(piv, dtype=np.int64)
    r = piv.size
    Li = np.asfortranarray(Linv, dtype=np.float64)
    dt = torch.float64 if p == KEVD_FP64 else torch.float32
    F = torch.empty((N, r), dtype=dt, device=X.device)
    ctx._check(ctx.lib.kevd_factor_from_linv(ctx.h, _ptr(X), N, d, float(scale), _np_ptr(piv), r,
                                             Li.ctypes.data, p, _ptr(F), r, _stream()))
    return F


def rpcholesky_batched(ctx: Context, Xs, scales, k_max, block=32, seeds=None, max_rounds=None,
                       use_graph: bool = True) -> list:
    """Mixed-precision block RPCholesky of many datasets at once
    (``kevd_rpchol_batched``): with ``use_graph`` every job's round loop is a
    branch of one captured CUDA graph launched once.  Returns one
    Factorization per job (FP32 factor)."""
    n = len(Xs)
    k_max = list(k_max) if hasattr(k_max, "__len__") else [int(k_max)] * n
    block = list(block) if hasattr(block, "__len__") else [int(block)] * n
    seeds = list(seeds) if seeds is not None else [1234 + q for q in range(n)]
    jobs = (_lib.RpcholJob * n)()
    Fs, pivs, mr = [], [], []
    for q, X in enumerate(Xs):
        _need_cuda(X, torch.float32, "X")
        N, d = X.shape
        F = torch.empty((N, k_max[q]), dtype=torch.float32, device=X.device)
        piv = np.zeros(k_max[q], dtype=np.int64)
        rounds = max_rounds[q] if max_rounds is not None else max(1, 4 * ((k_max[q] + block[q] - 1) // block[q]) + 8)
        Fs.append(F)
        pivs.append(piv)
        mr.append(rounds)
        jobs[q] = _lib.RpcholJob(X.data_ptr(), N, d, block[q], float(scales[q]), F.data_ptr(), k_max[q], k_max[q],
                                 rounds, 0, int(seeds[q]), piv.ctypes.data, _lib.RpcholResult())
    ctx._check(ctx.lib.kevd_rpchol_batched(ctx.h, jobs, n, 1 if use_graph else 0, _stream()))
    out = []
    for q in range(n):
        r = jobs[q].result
        out.append(Factorization(F=Fs[q], piv=pivs[q][: r.rank].copy(), err=np.zeros(0), accepted=np.zeros(0, np.int32),
                                 rank=int(r.rank), rounds=int(r.rounds), trace_error=float(r.trace_error),
                                 precision=KEVD_MIXED, scale=float(scales[q])))
    return out


def factor_from_pivots(ctx: Context, X: torch.Tensor, scale: float, piv, precision="fp64",
                       F: torch.Tensor | None = None) -> torch.Tensor:
    """F = K(:, S) L^{-T}, L L^T = K(S, S), in FP64 arithmetic for the given pivots."""
    _need_cuda(X, torch.float32, "X")
    N, d = X.shape
    p = _prec(precision)
    piv = np.ascontiguousarray(piv, dtype=np.int64)
    r = piv.size
    dt = torch.float64 if p == KEVD_FP64 else torch.float32
    if F is None:
        F = torch.empty((N, r), dtype=dt, device=X.device)
    ctx._check(ctx.lib.kevd_factor_from_pivots(ctx.h, _ptr(X), N, d, float(scale), _np_ptr(piv), r, p, _ptr(F),
                                               F.stride(0), _stream()))
    return F


# ---- stage 3 ---------------------------------------------------------------
@dataclass
class Eigendecomposition:
    lam: np.ndarray                 # k eigenvalues, ascending
    U: torch.Tensor                 # N x k_out float32, columns ascending
    trace_A: float
    shift: float
    dump: dict = field(default_factory=dict)


def bistochastic_evd(ctx: Context, F: torch.Tensor, k: int | None = None, k_out: int = 32,
                     precision=None, dump: bool = False, U: torch.Tensor | None = None) -> Eigendecomposition:
    if not (F.is_cuda and F.dtype in (torch.float32, torch.float64) and F.stride(1) == 1):
        raise ValueError("F must be a CUDA float32/float64 tensor with unit column stride")
    p = KEVD_FP64 if F.dtype == torch.float64 else KEVD_MIXED
    if precision is not None and _prec(precision) != p:
        raise ValueError("precision does not match F's dtype")
    N = F.shape[0]
    ldF = F.stride(0)
    if k is None:
        k = F.shape[1]
    lam = np.zeros(k, dtype=np.float64)
    if U is None:
        U = torch.empty((N, k_out), dtype=torch.float32, device=F.device)
    info = EvdInfo()
    dmp = None
    host = {}
    if dump:
        host = dict(c1=np.zeros(k), dtil=np.zeros(N), cq=np.zeros(k), qtil=np.zeros(N),
                    A=np.zeros((k, k), order="F"), B=np.zeros((k, k), order="F"),
                    W=np.zeros((k, k), order="F"), Z=np.zeros((k, k_out), order="F"))
        dmp = EvdDump(**{n: a.ctypes.data_as(C.POINTER(C.c_double)) for n, a in host.items()})
    ctx._check(ctx.lib.kevd_bistochastic_evd(ctx.h, _ptr(F), p, N, k, ldF, k_out, _np_ptr(lam), _ptr(U),
                                             C.byref(info), C.byref(dmp) if dmp is not None else None,
                                             _stream()))
    return Eigendecomposition(lam=lam, U=U, trace_A=info.trace_A, shift=info.shift, dump=host)


def weighted_gram(ctx: Context, F: torch.Tensor, s: torch.Tensor, k: int | None = None) -> torch.Tensor:
    """G = F^T diag(s)^2 F (k x k FP64 on the device; FP32 F runs on the tensor cores)."""
    if not (F.is_cuda and F.dtype in (torch.float32, torch.float64) and F.stride(1) == 1):
        raise ValueError("F must be a CUDA float32/float64 tensor with unit column stride")
    _need_cuda(s, torch.float64, "s")
    p = KEVD_FP64 if F.dtype == torch.float64 else KEVD_MIXED
    N = F.shape[0]
    if k is None:
        k = F.shape[1]
    G = torch.empty((k, k), dtype=torch.float64, device=F.device)
    ctx._check(ctx.lib.kevd_weighted_gram(ctx.h, _ptr(F), p, N, k, F.stride(0), _ptr(s), _ptr(G), _stream()))
    return G.T.contiguous()   # column-major storage -> row-major view


def weighted_gram2(ctx: Context, F: torch.Tensor, s: torch.Tensor, s2: torch.Tensor,
                   k: int | None = None) -> tuple[torch.Tensor, torch.Tensor]:
    """(F^T diag(s)^2 F, F^T diag(s2)^2 F) in one pass over F (FP32 F: one tensor-core kernel)."""
    if not (F.is_cuda and F.dtype in (torch.float32, torch.float64) and F.stride(1) == 1):
        raise ValueError("F must be a CUDA float32/float64 tensor with unit column stride")
    _need_cuda(s, torch.float64, "s")
    _need_cuda(s2, torch.float64, "s2")
    p = KEVD_FP64 if F.dtype == torch.float64 else KEVD_MIXED
    N = F.shape[0]
    if k is None:
        k = F.shape[1]
    G = torch.empty((k, k), dtype=torch.float64, device=F.device)
    G2 = torch.empty((k, k), dtype=torch.float64, device=F.device)
    ctx._check(ctx.lib.kevd_weighted_gram2(ctx.h, _ptr(F), p, N, k, F.stride(0), _ptr(s), _ptr(s2), _ptr(G),
                                           _ptr(G2), _stream()))
    return G.T.contiguous(), G2.T.contiguous()


class NystromModel:
    """Resident landmarks + eigenfunction coefficients for out-of-sample states."""

    def __init__(self, ctx: Context, X: torch.Tensor, fac: Factorization, k_out: int = 32):
        _need_cuda(X, torch.float32, "X")
        self.ctx = ctx
        N, d = X.shape
        self.d = d
        self.k_out = k_out
        h = C.c_void_p()
        piv = np.ascontiguousarray(fac.piv, dtype=np.int64)
        ctx._check(ctx.lib.kevd_nystrom_prepare(ctx.h, _ptr(X), N, d, fac.scale, _ptr(fac.F), fac.precision,
                                                fac.F.shape[1], _np_ptr(piv), fac.rank, k_out, C.byref(h),
                                                _stream()))
        self.h = h

    def __call__(self, Y: torch.Tensor, out: torch.Tensor | None = None) -> torch.Tensor:
        _need_cuda(Y, torch.float32, "Y")
        n = Y.shape[0]
        if out is None:
            out = torch.empty((n, self.k_out), dtype=torch.float32, device=Y.device)
        self.ctx._check(self.ctx.lib.kevd_nystrom_eval(self.ctx.h, self.h, _ptr(Y), n, _ptr(out), _stream()))
        return out

    def close(self):
        if getattr(self, "h", None):
            self.ctx.lib.kevd_model_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---- serving loop ------------------------------------------------------------
@dataclass
class RequestResult:
    status: int
    model_id: int
    latency_s: float
    queue_s: float
    batch_rows: int
    trace_error: float
    rank: int


def factorization_footprint(N: int, d: int, k: int, k_out: int = 32, precision="mixed") -> int:
    """Bytes the server charges against its HBM budget for one factorization."""
    return int(_lib.load().kevd_factorization_footprint(N, d, k, k_out, _prec(precision)))


def model_bytes(rank: int, d: int, k_out: int) -> int:
    """Bytes a resident Nystrom model is charged (landmarks + [Z'|p1'])."""
    return rank * (4 * d + 8 * (k_out + 1))


class Server:
    """Resident models on one GPU, factorizations admitted by HBM footprint,
    Nystrom queries batched as they arrive (``kevd_server_*``).

    ``submit_factorization`` copies X (host float32, N x d).  ``submit_query``
    keeps a reference to Y (host float32, n x d) and writes into ``out``
    (host float32, n x k_out) until ``wait`` returns for that request."""

    def __init__(self, device: int = 0, factor_workers: int = 2, max_query_batch: int = 8192,
                 hbm_budget_bytes: int = 200 << 30, batch_window_us: float = 0.0):
        self.lib = _lib.load()
        cfg = _lib.ServerConfig(device, factor_workers, max_query_batch, hbm_budget_bytes, batch_window_us)
        h = C.c_void_p()
        check(self.lib.kevd_server_create(C.byref(cfg), C.byref(h)))
        self.h = h
        self._keep = {}   # request id -> host arrays the server still reads or writes

    def submit_factorization(self, X: np.ndarray, scale: float, k: int, block: int = 64, k_out: int = 32,
                             seed: int = 0, precision="mixed") -> int:
        X = np.ascontiguousarray(X, dtype=np.float32)
        rid = C.c_int64()
        check(self.lib.kevd_server_submit_factorization(self.h, _np_ptr(X), X.shape[0], X.shape[1], float(scale),
                                                        int(k), int(block), int(k_out), int(seed),
                                                        _prec(precision), C.byref(rid)))
        return rid.value

    def submit_query(self, model_id: int, Y: np.ndarray, k_out: int) -> tuple[int, np.ndarray]:
        Y = np.ascontiguousarray(Y, dtype=np.float32)
        out = np.empty((Y.shape[0], k_out), dtype=np.float32)
        rid = C.c_int64()
        check(self.lib.kevd_server_submit_query(self.h, int(model_id), _np_ptr(Y), Y.shape[0], _np_ptr(out),
                                                C.byref(rid)))
        self._keep[rid.value] = (Y, out)
        return rid.value, out

    def wait(self, rid: int, timeout_s: float = 600.0) -> RequestResult:
        info = _lib.RequestInfo()
        check(self.lib.kevd_server_wait(self.h, int(rid), float(timeout_s), C.byref(info)))
        self._keep.pop(rid, None)
        res = RequestResult(info.status, info.model_id, info.latency_s, info.queue_s, info.batch_rows,
                            info.trace_error, info.rank)
        if res.status != 0:
            raise KevdError(res.status, f"request {rid} failed: {info.message.decode(errors='replace')}")
        return res

    def release_model(self, model_id: int):
        check(self.lib.kevd_server_release_model(self.h, int(model_id)))

    def stats(self, kind: str) -> dict:
        p50, p99, n = C.c_double(), C.c_double(), C.c_int64()
        check(self.lib.kevd_server_stats(self.h, {"factorization": 0, "query": 1}[kind], C.byref(p50),
                                         C.byref(p99), C.byref(n)))
        return {"p50_s": p50.value, "p99_s": p99.value, "count": n.value}

    def memory(self) -> dict:
        used, act, mods, peak = C.c_int64(), C.c_int32(), C.c_int32(), C.c_int32()
        check(self.lib.kevd_server_memory(self.h, C.byref(used), C.byref(act), C.byref(mods), C.byref(peak)))
        return {"used_bytes": used.value, "active": act.value, "models": mods.value, "peak_active": peak.value}

    def close(self):
        if getattr(self, "h", None):
            self.lib.kevd_server_destroy(self.h)
            self.h = None
            self._keep.clear()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---- profiling ---------------------------------------------------------------
def profile_enable(ctx: Context, on: bool = True):
    """Record per-kernel device time (CUDA events on the launching stream)."""
    ctx._check(ctx.lib.kevd_profile_enable(ctx.h, 1 if on else 0))


def profile_read(ctx: Context) -> dict:
    """{kernel name: (total ms, launches)} accumulated since profile_enable."""
    out = {}
    buf = C.create_string_buffer(128)
    i = 0
    while True:
        ms = C.c_double()
        cnt = C.c_int64()
        st = ctx.lib.kevd_profile_read(ctx.h, i, buf, 128, C.byref(ms), C.byref(cnt))
        if st != 0:
            break
        out[buf.value.decode()] = (ms.value, cnt.value)
        i += 1
    return out


def peak_rate(ctx: Context, kind: str) -> dict:
    """Measured issue rate: kind "ex2" (MUFU ex2/s), "fp32_fma", "fp64_fma" or
    "fp32x2_fma" (FMA/s; the last issued as packed FP32 pairs)."""
    k = {"ex2": 0, "fp32_fma": 1, "fp64_fma": 2, "fp32x2_fma": 3}[kind]
    rate, ms = C.c_double(), C.c_double()
    ctx._check(ctx.lib.kevd_peak_rate(ctx.h, k, C.byref(rate), C.byref(ms), _stream()))
    return {"ops_per_s": rate.value, "ms": ms.value}


def launch_count(ctx: Context) -> int:
    """Kernels launched by this library through ctx so far."""
    return int(ctx.lib.kevd_launch_count(ctx.h))
