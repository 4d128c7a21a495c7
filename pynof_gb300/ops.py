"""Device-resident operations over torch CUDA tensors.

Each function allocates its outputs with torch, takes scratch from a per-device
workspace pool, and calls one C-ABI entry point of ``libpynof_gb300.so`` on
torch's current CUDA stream.  torch supplies memory and streams only; all
arithmetic is in the library's CUDA kernels.  Inputs must already be float64
CUDA tensors (``to_device`` converts numpy arrays).
"""
from __future__ import annotations

import ctypes
import threading

import numpy as np
import torch

from . import _lib

_F64 = torch.float64


def _ptr(t: torch.Tensor | None) -> int | None:
    return None if t is None else t.data_ptr()


def _stream(device: torch.device | None = None) -> int:
    return torch.cuda.current_stream(device).cuda_stream


def to_device(x, device=None) -> torch.Tensor:
    """float64, C-contiguous CUDA tensor view/copy of ``x`` (numpy or torch)."""
    device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
    if isinstance(x, torch.Tensor):
        t = x.to(device=device, dtype=_F64)
    else:
        t = torch.from_numpy(np.ascontiguousarray(np.asarray(x, dtype=np.float64))).to(device)
    return t.contiguous()


def _require(t: torch.Tensor, shape, name: str) -> None:
    if not isinstance(t, torch.Tensor) or not t.is_cuda:
        raise TypeError(f"{name} must be a CUDA tensor")
    if t.dtype != _F64:
        raise TypeError(f"{name} must be float64, got {t.dtype}")
    if tuple(t.shape) != tuple(shape):
        raise ValueError(f"{name} has shape {tuple(t.shape)}, expected {tuple(shape)}")
    if not t.is_contiguous():
        raise ValueError(f"{name} must be contiguous")


class WorkspacePool:
    """One growing scratch buffer per (device, stream); reused across calls.

    Calls on the same stream are ordered, so reuse is safe; different streams
    get different buffers.
    """

    def __init__(self):
        self._bufs: dict[tuple[int, int], torch.Tensor] = {}
        self._lock = threading.Lock()

    def get(self, nbytes: int, device: torch.device) -> torch.Tensor:
        key = (device.index if device.index is not None else torch.cuda.current_device(), _stream(device))
        with self._lock:
            buf = self._bufs.get(key)
            if buf is None or buf.numel() < nbytes:
                buf = torch.empty(max(nbytes, 256), dtype=torch.uint8, device=device)
                self._bufs[key] = buf
            return buf

    def clear(self) -> None:
        with self._lock:
            self._bufs.clear()


POOL = WorkspacePool()


def _ws(query: str, *sizes, device) -> tuple[int, int]:
    n = _lib.query(query, *sizes)
    buf = POOL.get(n, device)
    return buf.data_ptr(), buf.numel()


# ----------------------------------------------------------------------------
def check_symmetric(b: torch.Tensor) -> float:
    """max |b[m, n, l] - b[n, m, l]| (the RI kernels require exact symmetry)."""
    N, N2, Q = b.shape
    _require(b, (N, N, Q), "b")
    out = torch.empty(1, dtype=_F64, device=b.device)
    _lib.call("gb_check_symmetric_f64", _ptr(b), N, Q, _ptr(out), _stream(b.device))
    return float(out.item())


def jkj_ri(C: torch.Tensor, b: torch.Tensor, nbf5: int):
    """J, K (nbf5, nbf, nbf) from the RI factor (A1, computeJKj)."""
    N, _, Q = b.shape
    _require(C, (N, N), "C")
    _require(b, (N, N, Q), "b")
    J = torch.empty((nbf5, N, N), dtype=_F64, device=b.device)
    K = torch.empty((nbf5, N, N), dtype=_F64, device=b.device)
    wp, wn = _ws("gb_jkj_ri_workspace_f64", N, nbf5, Q, device=b.device)
    _lib.call("gb_jkj_ri_f64", _ptr(C), _ptr(b), N, nbf5, Q, _ptr(J), _ptr(K), wp, wn, _stream(b.device))
    return J, K


def _outs(out, shapes, dev):
    """Caller-provided output tensors (checked) or new ones."""
    if out is None:
        return [torch.empty(sh, dtype=_F64, device=dev) for sh in shapes]
    for t, sh in zip(out, shapes):
        _require(t, sh, "out")
    return list(out)


def jkh_mo_ri(C: torch.Tensor, H: torch.Tensor, b: torch.Tensor, nbf5: int, out=None):
    """J_MO, K_MO (nbf5, nbf5), H_core (nbf5,) from the RI factor (A3)."""
    N, _, Q = b.shape
    _require(C, (N, N), "C")
    _require(H, (N, N), "H")
    _require(b, (N, N, Q), "b")
    dev = b.device
    J_MO, K_MO, H_core = _outs(out, [(nbf5, nbf5), (nbf5, nbf5), (nbf5,)], dev)
    wp, wn = _ws("gb_jkh_mo_ri_workspace_f64", N, nbf5, Q, device=dev)
    _lib.call("gb_jkh_mo_ri_f64", _ptr(C), _ptr(H), _ptr(b), N, nbf5, Q, _ptr(J_MO), _ptr(K_MO), _ptr(H_core),
              wp, wn, _stream(dev))
    return J_MO, K_MO, H_core


def mo_ri(C: torch.Tensor, H: torch.Tensor, b: torch.Tensor, nbf5: int):
    """Hmat (nbf, nbf5) and bMO (nbf, nbf5, naux) (A5, Integrals_MO_RI)."""
    N, _, Q = b.shape
    _require(C, (N, N), "C")
    _require(H, (N, N), "H")
    _require(b, (N, N, Q), "b")
    dev = b.device
    Hmat = torch.empty((N, nbf5), dtype=_F64, device=dev)
    bMO = torch.empty((N, nbf5, Q), dtype=_F64, device=dev)
    wp, wn = _ws("gb_mo_ri_workspace_f64", N, nbf5, Q, device=dev)
    _lib.call("gb_mo_ri_f64", _ptr(C), _ptr(H), _ptr(b), N, nbf5, Q, _ptr(Hmat), _ptr(bMO), wp, wn, _stream(dev))
    return Hmat, bMO


def lagrange2_ri(C, H, b, n, cj12, ck12, nbf5: int, nbeta: int, nalpha: int, out=None):
    """elag (nbf, nbf) and Hmat (nbf, nbf5) (A5, computeLagrange2 RI closed shell).

    The diagonals of cj12 / ck12 are ignored (treated as zero)."""
    N, _, Q = b.shape
    _require(C, (N, N), "C")
    _require(H, (N, N), "H")
    _require(b, (N, N, Q), "b")
    _require(n, (nbf5,), "n")
    _require(cj12, (nbf5, nbf5), "cj12")
    _require(ck12, (nbf5, nbf5), "ck12")
    dev = b.device
    elag, Hmat = _outs(out, [(N, N), (N, nbf5)], dev)
    wp, wn = _ws("gb_lagrange2_ri_workspace_f64", N, nbf5, Q, device=dev)
    _lib.call("gb_lagrange2_ri_f64", _ptr(C), _ptr(H), _ptr(b), _ptr(n), _ptr(cj12), _ptr(ck12), N, nbf5, Q,
              nbeta, nalpha, _ptr(elag), _ptr(Hmat), wp, wn, _stream(dev))
    return elag, Hmat


# ----------------------------------------------------------------------------
# full-ERI path (A2, A4, A6)
# ----------------------------------------------------------------------------
def jkj_full(C, I, nbf5: int):
    """J, K (nbf5, nbf, nbf) from the 4-index tensor (A2)."""
    N = C.shape[0]
    _require(C, (N, N), "C")
    _require(I, (N, N, N, N), "I")
    dev = I.device
    J = torch.empty((nbf5, N, N), dtype=_F64, device=dev)
    K = torch.empty((nbf5, N, N), dtype=_F64, device=dev)
    wp, wn = _ws("gb_jkj_full_workspace_f64", N, nbf5, device=dev)
    _lib.call("gb_jkj_full_f64", _ptr(C), _ptr(I), N, nbf5, _ptr(J), _ptr(K), wp, wn, _stream(dev))
    return J, K


def jkh_mo_full(C, H, I, nbf5: int):
    """J_MO, K_MO, H_core from the 4-index tensor (A4)."""
    N = C.shape[0]
    _require(C, (N, N), "C")
    _require(H, (N, N), "H")
    _require(I, (N, N, N, N), "I")
    dev = I.device
    J_MO = torch.empty((nbf5, nbf5), dtype=_F64, device=dev)
    K_MO = torch.empty((nbf5, nbf5), dtype=_F64, device=dev)
    H_core = torch.empty((nbf5,), dtype=_F64, device=dev)
    wp, wn = _ws("gb_jkh_mo_full_workspace_f64", N, nbf5, device=dev)
    _lib.call("gb_jkh_mo_full_f64", _ptr(C), _ptr(H), _ptr(I), N, nbf5, _ptr(J_MO), _ptr(K_MO), _ptr(H_core), wp, wn,
              _stream(dev))
    return J_MO, K_MO, H_core


def mo_full(C, H, I, nbf5: int):
    """Hmat (nbf, nbf5), I_MO (nbf, nbf5, nbf5, nbf5) (A6)."""
    N = C.shape[0]
    _require(C, (N, N), "C")
    _require(H, (N, N), "H")
    _require(I, (N, N, N, N), "I")
    dev = I.device
    Hmat = torch.empty((N, nbf5), dtype=_F64, device=dev)
    imo = torch.empty((N, nbf5, nbf5, nbf5), dtype=_F64, device=dev)
    wp, wn = _ws("gb_mo_full_workspace_f64", N, nbf5, device=dev)
    _lib.call("gb_mo_full_f64", _ptr(C), _ptr(H), _ptr(I), N, nbf5, _ptr(Hmat), _ptr(imo), wp, wn, _stream(dev))
    return Hmat, imo


def lagrange2_full(C, H, I, n, cj12, ck12, nbf5: int, nbeta: int, nalpha: int):
    """elag (nbf, nbf), Hmat (nbf, nbf5) from the 4-index tensor (A6)."""
    N = C.shape[0]
    _require(C, (N, N), "C")
    _require(H, (N, N), "H")
    _require(I, (N, N, N, N), "I")
    _require(n, (nbf5,), "n")
    _require(cj12, (nbf5, nbf5), "cj12")
    _require(ck12, (nbf5, nbf5), "ck12")
    dev = I.device
    elag = torch.empty((N, N), dtype=_F64, device=dev)
    Hmat = torch.empty((N, nbf5), dtype=_F64, device=dev)
    wp, wn = _ws("gb_lagrange2_full_workspace_f64", N, nbf5, device=dev)
    _lib.call("gb_lagrange2_full_f64", _ptr(C), _ptr(H), _ptr(I), _ptr(n), _ptr(cj12), _ptr(ck12), N, nbf5, nbeta,
              nalpha, _ptr(elag), _ptr(Hmat), wp, wn, _stream(dev))
    return elag, Hmat


# ----------------------------------------------------------------------------
# AO route: generalized Fock, Lagrangian, energy (A8, A7)
# ----------------------------------------------------------------------------
def fock_rc(J, K, n, H, cj12, ck12, nbeta: int, nalpha: int, no1: int = 0):
    """F (nbf5, nbf, nbf), closed shell (computeF_RC)."""
    P, N, _ = J.shape
    _require(J, (P, N, N), "J")
    _require(K, (P, N, N), "K")
    _require(n, (P,), "n")
    _require(H, (N, N), "H")
    _require(cj12, (P, P), "cj12")
    _require(ck12, (P, P), "ck12")
    dev = J.device
    F = torch.empty((P, N, N), dtype=_F64, device=dev)
    wp, wn = _ws("gb_fock_rc_workspace_f64", N, P, device=dev)
    _lib.call("gb_fock_rc_f64", _ptr(J), _ptr(K), _ptr(n), _ptr(H), _ptr(cj12), _ptr(ck12), N, P, nbeta, nalpha, no1,
              _ptr(F), wp, wn, _stream(dev))
    return F


def fock_ro(J, K, n, H, cj12, ck12, nbeta: int, nalpha: int, no1: int = 0):
    """F (nbf5, nbf, nbf), restricted open shell (computeF_RO)."""
    P, N, _ = J.shape
    _require(J, (P, N, N), "J")
    _require(K, (P, N, N), "K")
    _require(n, (P,), "n")
    _require(H, (N, N), "H")
    _require(cj12, (P, P), "cj12")
    _require(ck12, (P, P), "ck12")
    dev = J.device
    F = torch.empty((P, N, N), dtype=_F64, device=dev)
    wp, wn = _ws("gb_fock_ro_workspace_f64", N, P, device=dev)
    _lib.call("gb_fock_ro_f64", _ptr(J), _ptr(K), _ptr(n), _ptr(H), _ptr(cj12), _ptr(ck12), N, P, nbeta, nalpha, no1,
              _ptr(F), wp, wn, _stream(dev))
    return F


def lagrange(F, C, noptorb: int | None = None):
    """elag (nbf, nbf) from the generalized Fock matrices (computeLagrange)."""
    P, N, _ = F.shape
    _require(F, (P, N, N), "F")
    _require(C, (N, N), "C")
    dev = F.device
    elag = torch.empty((N, N), dtype=_F64, device=dev)
    wp, wn = _ws("gb_lagrange_workspace_f64", N, P, device=dev)
    _lib.call("gb_lagrange_f64", _ptr(F), _ptr(C), N, P, noptorb or N, _ptr(elag), wp, wn, _stream(dev))
    return elag


def energy_elec(elag, C, H, n, nbeta: int, nalpha: int, high_spin: bool = False):
    """Electronic energy (computeE_elec) as a 0-d CUDA tensor."""
    N = C.shape[0]
    P = n.shape[0]
    _require(elag, (N, N), "elag")
    _require(C, (N, N), "C")
    _require(H, (N, N), "H")
    _require(n, (P,), "n")
    dev = C.device
    E = torch.empty((), dtype=_F64, device=dev)
    wp, wn = _ws("gb_energy_elec_workspace_f64", N, P, device=dev)
    _lib.call("gb_energy_elec_f64", _ptr(elag), _ptr(C), _ptr(H), _ptr(n), N, P, nbeta, nalpha, int(high_spin),
              _ptr(E), wp, wn, _stream(dev))
    return E


def ri_factor(mnk: torch.Tensor, M: torch.Tensor, nslices: int | None = None) -> torch.Tensor:
    """b[m][n][l] = sum_k mnk[m][n][k] M[k][l] (M symmetric): FP64 DMMA, or the
    split-product tensor-core GEMM when ``nslices`` is given."""
    N, N2, Q = mnk.shape
    if N2 != N:
        raise ValueError("mnk must be (nbf, nbf, naux)")
    _require(mnk, (N, N, Q), "mnk")
    _require(M, (Q, Q), "M")
    if nslices is not None:
        return dgemm_mixed(mnk.view(N * N, Q), M, nslices).view(N, N, Q)
    b = torch.empty((N, N, Q), dtype=_F64, device=mnk.device)
    _lib.call("gb_ri_factor_f64", _ptr(mnk), _ptr(M), N, Q, _ptr(b), _stream(mnk.device))
    return b


def mo4_full(C: torch.Tensor, I: torch.Tensor, p, q, r, t) -> torch.Tensor:
    """out[p][q][r][t] = sum C[m,p] C[n,q] I[m,n,s,l] C[s,r] C[l,t] over the
    orbital ranges p, q, r, t (each a (start, stop) pair)."""
    N = C.shape[0]
    _require(C, (N, N), "C")
    _require(I, (N, N, N, N), "I")
    (p0, p1), (q0, q1), (r0, r1), (t0, t1) = p, q, r, t
    out = torch.empty((p1 - p0, q1 - q0, r1 - r0, t1 - t0), dtype=_F64, device=C.device)
    wp, wn = _ws("gb_mo4_full_workspace_f64", N, q1 - q0, r1 - r0, t1 - t0, device=C.device)
    _lib.call("gb_mo4_full_f64", _ptr(C), _ptr(I), N, p0, p1 - p0, q0, q1 - q0, r0, r1 - r0, t0, t1 - t0,
              _ptr(out), wp, wn, _stream(C.device))
    return out


def density_hf(C: torch.Tensor, j0: int, j1: int) -> torch.Tensor:
    """D = sum_{j0 <= j < j1} C[:, j] C[:, j]^T (computeD_HF / computeDalpha_HF)."""
    N = C.shape[0]
    _require(C, (N, N), "C")
    D = torch.empty((N, N), dtype=_F64, device=C.device)
    _lib.call("gb_density_hf_f64", _ptr(C), N, int(j0), int(j1), _ptr(D), _stream(C.device))
    return D


def jk_hf_full(D: torch.Tensor, I: torch.Tensor):
    """J, K of one symmetric density from the 4-index tensor (JK_HF_Full_GPU)."""
    N = D.shape[0]
    _require(D, (N, N), "D")
    _require(I, (N, N, N, N), "I")
    J = torch.empty((N, N), dtype=_F64, device=D.device)
    K = torch.empty((N, N), dtype=_F64, device=D.device)
    wp, wn = _ws("gb_jk_hf_full_workspace_f64", N, device=D.device)
    _lib.call("gb_jk_hf_full_f64", _ptr(D), _ptr(I), N, _ptr(J), _ptr(K), wp, wn, _stream(D.device))
    return J, K


def rotate_orbital(y: torch.Tensor, C: torch.Tensor, nbf5: int, out: torch.Tensor | None = None,
                   norm1: float = -1.0) -> torch.Tensor:
    """C expm(Y) (rotate_orbital) with Y the antisymmetric matrix of the packed
    step y (rows i < nbf5 of the strict upper triangle, row-major).

    norm1: an upper bound of ||Y||_1 (see :func:`antisym_norm1`); negative
    means "measure it on the device" (one stream synchronisation)."""
    N = C.shape[0]
    _require(C, (N, N), "C")
    nvar = N * (N - 1) // 2 - (N - nbf5) * (N - nbf5 - 1) // 2
    _require(y, (nvar,), "y")
    dev = C.device
    if out is None:
        out = torch.empty_like(C)
    else:
        _require(out, (N, N), "out")
    wp, wn = _ws("gb_rotate_orbital_workspace_f64", N, device=dev)
    _lib.call("gb_rotate_orbital_f64", _ptr(y), _ptr(C), N, nbf5, float(norm1), _ptr(out), wp, wn, _stream(dev))
    return out


class OccMinimizer:
    """occoptr's minimisation of the occupation energy over gamma on the
    device (``gb_occ_minimize_dev``; ``pynof/minimization.py:77-97``): scipy's
    CG (Polak-Ribiere+, More-Thuente line search, gtol 1e-5 on ||g||_inf) over
    E(gamma) of calcocce / calcoccg at fixed device J_MO, K_MO, H_core, as one
    CUDA graph per minimisation with no host synchronisation.  Owns its
    workspace (the library caches the graph per workspace) and its outputs;
    one minimisation at a time per object, on the current stream."""

    def __init__(self, nbf5: int, no1: int, ndoc: int, ncwo: int, device=None):
        self.dims = (int(nbf5), int(no1), int(ndoc), int(ncwo))
        self.nv = ndoc * ncwo
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        self._wn = _lib.query("gb_occ_workspace_bytes", nbf5, ndoc, ncwo)
        if self._wn == 0:
            raise ValueError(f"no occupation problem for nbf5={nbf5}, ndoc={ndoc}, ncwo={ncwo}")
        self._ws = torch.empty(self._wn + 256, dtype=torch.uint8, device=self.device)
        self._wp = (self._ws.data_ptr() + 255) & ~255

        def z(*shape):
            return torch.zeros(shape, dtype=_F64, device=self.device)

        self.result = z(5)  # E, iterations, evaluations, success, ||g||_inf
        self.gamma = z(self.nv)
        self.grad = z(self.nv)
        self.n = z(nbf5)
        self.cj12 = z(nbf5, nbf5)
        self.ck12 = z(nbf5, nbf5)

    def _check(self, gamma, J, K, H):
        P = self.dims[0]
        _require(gamma, (self.nv,), "gamma")
        _require(J, (P, P), "J_MO")
        _require(K, (P, P), "K_MO")
        _require(H, (P,), "H_core")

    def minimize(self, gamma0, J_MO, K_MO, H_core, gtol: float = 1e-5, maxiter: int | None = None,
                 coefficients: bool = True, host_driven: bool = False):
        """Launch the minimisation from gamma0; returns the device tensors
        (gamma, result, n, cj12, ck12) it fills (n, cj12, ck12 at the result;
        None with ``coefficients=False``).  ``host_driven`` replays an
        ordinary graph of eight evaluations and reads the phase back after
        each (``gb_occ_minimize_dev_sync``; returns when done) instead of the
        conditional-node graph."""
        self._check(gamma0, J_MO, K_MO, H_core)
        maxiter = 200 * self.nv if maxiter is None else int(maxiter)
        co = (self.n, self.cj12, self.ck12) if coefficients else (None, None, None)
        entry = "gb_occ_minimize_dev_sync" if host_driven else "gb_occ_minimize_dev"
        _lib.call(entry, _ptr(gamma0), _ptr(J_MO), _ptr(K_MO), _ptr(H_core), *self.dims,
                  float(gtol), maxiter, _ptr(self.gamma), _ptr(self.result), *(_ptr(t) for t in co), self._wp,
                  self._wn, _stream(self.device))
        return (self.gamma, self.result) + co

    def energy_grad(self, gamma, J_MO, K_MO, H_core):
        """One evaluation: (result, grad) device tensors, result[0] = E."""
        self._check(gamma, J_MO, K_MO, H_core)
        _lib.call("gb_occ_energy_grad_dev", _ptr(gamma), _ptr(J_MO), _ptr(K_MO), _ptr(H_core), *self.dims,
                  _ptr(self.result), _ptr(self.grad), self._wp, self._wn, _stream(self.device))
        return self.result, self.grad

    def close(self) -> None:
        """Drop the library's cached graphs for this workspace.  A graph still
        running is freed when it completes (cudaGraphExecDestroy), and the
        workspace memory returns to torch's allocator in stream order, so no
        synchronisation is needed -- in a server, a device-wide one would wait
        for every other request's work."""
        if self._ws is not None:
            _lib.call("gb_occ_release", self._wp)
            self._ws = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class StreamGraph:
    """Work issued by this thread on ``stream`` between ``begin`` and ``end``,
    captured (thread-local mode) into a CUDA graph and replayed by
    ``launch``.  The captured work must not allocate or synchronise: give the
    ops preallocated outputs and grow their workspaces in a run beforehand."""

    def __init__(self, stream):
        self.stream = stream
        self.handle = ctypes.c_void_p()

    def begin(self):
        _lib.call("gb_graph_begin", self.stream.cuda_stream)

    def end(self):
        _lib.call("gb_graph_end", self.stream.cuda_stream, ctypes.byref(self.handle))

    def launch(self):
        _lib.call("gb_graph_launch", self.handle, self.stream.cuda_stream)

    def __del__(self):
        if self.handle:
            try:
                _lib.call("gb_graph_destroy", self.handle)
            except Exception:  # interpreter shutdown
                pass
            self.handle = ctypes.c_void_p()


class AntisymNorm:
    """||Y||_1 (max column sum of |Y|) of the antisymmetric matrix of a packed
    step, on the host from y alone (index arrays built once per size)."""

    def __init__(self, nbf: int, nbf5: int):
        iu, ju = np.triu_indices(nbf, 1)
        keep = iu < nbf5
        self.iu, self.ju, self.n = iu[keep], ju[keep], nbf

    def __call__(self, y) -> float:
        a = np.abs(np.asarray(y, dtype=np.float64))
        col = np.bincount(self.iu, a, minlength=self.n) + np.bincount(self.ju, a, minlength=self.n)
        return float(col.max()) if col.size else 0.0


# ----------------------------------------------------------------------------
# split-product tensor-core path
# ----------------------------------------------------------------------------
_STATUS_MESSAGES = {
    5: "a tensor-core kernel gave up on a bounded wait; its outputs (and those of every split-product call "
       "since) are not valid",
    6: "an operand of a split-product call held a NaN or an infinity; the outputs are not valid",
}


def check_device_status(reset: bool = False) -> None:
    """Raise GBError if a tensor-core kernel recorded an error on the current
    device (GB_ERR_TIMEOUT, GB_ERR_NONFINITE).  Synchronises the device.

    The status word is shared by every caller on the device and stays set
    until :func:`reset_device_status` (or ``reset=True`` here) clears it, so a
    failure is reported to every caller that checks after its own work rather
    than to whichever checks first."""
    st = _lib.device_status(reset=reset)
    if st != 0:
        raise _lib.GBError(st, _STATUS_MESSAGES.get(st, "tensor-core status word is set"))


def reset_device_status() -> int:
    """Clear the tensor-core status word; returns what it held."""
    return _lib.device_status(reset=True)


#: Split code of the three-product TF32 form (``GB_SPLIT_TF32X3``), accepted
#: wherever ``nslices`` is (1..6 select bf16 digit slices).
SPLIT_TF32X3 = 32


def dgemm_mixed(A: torch.Tensor, B: torch.Tensor, nslices: int = 6) -> torch.Tensor:
    """C = A B^T (FP64-accurate at nslices=6) on the tcgen05 tensor cores."""
    M, K = A.shape
    N, K2 = B.shape
    if K2 != K:
        raise ValueError("A and B must share K")
    _require(A, (M, K), "A")
    _require(B, (N, K), "B")
    C = torch.empty((M, N), dtype=_F64, device=A.device)
    wp, wn = _ws("gb_dgemm_mixed_workspace", M, N, K, nslices, device=A.device)
    _lib.call("gb_dgemm_mixed", _ptr(A), _ptr(B), M, N, K, nslices, _ptr(C), wp, wn, _stream(A.device))
    return C


def dgemm_f64(A: torch.Tensor, B: torch.Tensor) -> torch.Tensor:
    """C = A B^T in FP64 on the DMMA engine."""
    M, K = A.shape
    N, K2 = B.shape
    if K2 != K:
        raise ValueError("A and B must share K")
    _require(A, (M, K), "A")
    _require(B, (N, K), "B")
    C = torch.empty((M, N), dtype=_F64, device=A.device)
    _lib.call("gb_dgemm_f64", _ptr(A), _ptr(B), M, N, K, _ptr(C), _stream(A.device))
    return C


class PreparedRI:
    """RI factor sliced for the tensor-core path (resident next to b)."""

    def __init__(self, b: torch.Tensor, nslices: int = 6):
        N, _, Q = b.shape
        _require(b, (N, N, Q), "b")
        self.nbf, self.naux, self.nslices = N, Q, nslices
        nbytes = _lib.query("gb_ri_prepare_bytes_mixed", N, Q, nslices)
        self.buf = torch.empty(nbytes, dtype=torch.uint8, device=b.device)
        _lib.call("gb_ri_prepare_mixed", _ptr(b), N, Q, nslices, self.buf.data_ptr(), nbytes, _stream(b.device))

    @property
    def device(self):
        return self.buf.device


def jkj_ri_mixed(C: torch.Tensor, prep: PreparedRI, nbf5: int):
    """J, K (nbf5, nbf, nbf) on the tensor cores (A1, computeJKj)."""
    N, Q, S = prep.nbf, prep.naux, prep.nslices
    _require(C, (N, N), "C")
    dev = prep.device
    J = torch.empty((nbf5, N, N), dtype=_F64, device=dev)
    K = torch.empty((nbf5, N, N), dtype=_F64, device=dev)
    wp, wn = _ws("gb_jkj_ri_workspace_mixed", N, nbf5, Q, S, device=dev)
    _lib.call("gb_jkj_ri_mixed", _ptr(C), prep.buf.data_ptr(), N, nbf5, Q, S, _ptr(J), _ptr(K), wp, wn,
              _stream(dev))
    return J, K


_COPY_STREAMS: dict = {}
_COPY_LOCK = threading.Lock()


def _copy_stream(dev: torch.device, main: torch.cuda.Stream) -> torch.cuda.Stream:
    """A second stream for the device-to-host copies of work on ``main`` (one
    per compute stream, so concurrent callers on their own streams never
    wait on each other's copies)."""
    key = (dev, main.cuda_stream)
    with _COPY_LOCK:
        s = _COPY_STREAMS.get(key)
        if s is None:
            s = _COPY_STREAMS[key] = torch.cuda.Stream(device=dev)
        return s


def jkj_ri_mixed_host(C: torch.Tensor, prep: PreparedRI, nbf5: int, block: int = 128):
    """J, K (nbf5, nbf, nbf) as numpy arrays in pinned host memory, with the
    device-to-host copies overlapped with the build.  The build runs as its
    prelude (T, d: ``gb_jkj_ri_mixed_t``), then J and K over alternating
    ranges of ``block`` orbitals (a multiple of 128: ``gb_jkj_ri_mixed_jr`` /
    ``gb_jkj_ri_mixed_k``); each range is copied on a second stream as soon as
    it is done, so the copies run back to back from shortly after T is formed.
    Bitwise the results of :func:`jkj_ri_mixed`."""
    N, Q, S = prep.nbf, prep.naux, prep.nslices
    _require(C, (N, N), "C")
    if block < 128 or block % 128:
        raise ValueError("block must be a positive multiple of 128")
    dev = prep.device
    J = torch.empty((nbf5, N, N), dtype=_F64, device=dev)
    K = torch.empty((nbf5, N, N), dtype=_F64, device=dev)
    Jh = torch.empty((nbf5, N, N), dtype=_F64, pin_memory=True)
    Kh = torch.empty((nbf5, N, N), dtype=_F64, pin_memory=True)
    wp, wn = _ws("gb_jkj_ri_workspace_mixed", N, nbf5, Q, S, device=dev)
    main = torch.cuda.current_stream(dev)
    cs = _copy_stream(dev, main)
    _lib.call("gb_jkj_ri_mixed_t", _ptr(C), prep.buf.data_ptr(), N, nbf5, Q, S, wp, wn, main.cuda_stream)
    for q0 in range(0, nbf5, block):
        q1 = min(q0 + block, nbf5)
        _lib.call("gb_jkj_ri_mixed_jr", prep.buf.data_ptr(), N, nbf5, Q, S, q0, q1, _ptr(J), wp, wn,
                  main.cuda_stream)
        cs.wait_stream(main)
        with torch.cuda.stream(cs):
            Jh[q0:q1].copy_(J[q0:q1], non_blocking=True)
        _lib.call("gb_jkj_ri_mixed_k", N, nbf5, Q, S, q0, q1, _ptr(K), wp, wn, main.cuda_stream)
        cs.wait_stream(main)
        with torch.cuda.stream(cs):
            Kh[q0:q1].copy_(K[q0:q1], non_blocking=True)
    cs.synchronize()
    check_device_status()
    return Jh.numpy(), Kh.numpy()


def jkh_mo_ri_mixed(C, H, prep: PreparedRI, nbf5: int, out=None):
    """J_MO, K_MO, H_core on the tensor cores (A3)."""
    N, Q, S = prep.nbf, prep.naux, prep.nslices
    _require(C, (N, N), "C")
    _require(H, (N, N), "H")
    dev = prep.device
    J_MO, K_MO, H_core = _outs(out, [(nbf5, nbf5), (nbf5, nbf5), (nbf5,)], dev)
    wp, wn = _ws("gb_jkh_mo_ri_workspace_mixed", N, nbf5, Q, S, device=dev)
    _lib.call("gb_jkh_mo_ri_mixed", _ptr(C), _ptr(H), prep.buf.data_ptr(), N, nbf5, Q, S, _ptr(J_MO), _ptr(K_MO),
              _ptr(H_core), wp, wn, _stream(dev))
    return J_MO, K_MO, H_core


def lagrange2_ri_mixed(C, H, prep: PreparedRI, n, cj12, ck12, nbf5: int, nbeta: int, nalpha: int, out=None):
    """elag, Hmat on the tensor cores (A5, closed shell)."""
    N, Q, S = prep.nbf, prep.naux, prep.nslices
    _require(C, (N, N), "C")
    _require(H, (N, N), "H")
    _require(n, (nbf5,), "n")
    _require(cj12, (nbf5, nbf5), "cj12")
    _require(ck12, (nbf5, nbf5), "ck12")
    dev = prep.device
    elag, Hmat = _outs(out, [(N, N), (N, nbf5)], dev)
    wp, wn = _ws("gb_lagrange2_ri_workspace_mixed", N, nbf5, Q, S, device=dev)
    _lib.call("gb_lagrange2_ri_mixed", _ptr(C), _ptr(H), prep.buf.data_ptr(), _ptr(n), _ptr(cj12), _ptr(ck12), N,
              nbf5, Q, nbeta, nalpha, S, _ptr(elag), _ptr(Hmat), wp, wn, _stream(dev))
    return elag, Hmat


def jkh_lagrange2_ri_mixed(C, H, prep: PreparedRI, n, cj12, ck12, nbf5: int, nbeta: int, nalpha: int, out=None):
    """computeJKH_MO and computeLagrange2 at the same orbitals in one call on
    the tensor cores (one half transform and one MO transform serve both):
    (J_MO, K_MO, H_core, elag, Hmat)."""
    N, Q, S = prep.nbf, prep.naux, prep.nslices
    _require(C, (N, N), "C")
    _require(H, (N, N), "H")
    _require(n, (nbf5,), "n")
    _require(cj12, (nbf5, nbf5), "cj12")
    _require(ck12, (nbf5, nbf5), "ck12")
    dev = prep.device
    J_MO, K_MO, H_core, elag, Hmat = _outs(out, [(nbf5, nbf5), (nbf5, nbf5), (nbf5,), (N, N), (N, nbf5)], dev)
    wp, wn = _ws("gb_jkh_lagrange2_ri_workspace_mixed", N, nbf5, Q, S, device=dev)
    _lib.call("gb_jkh_lagrange2_ri_mixed", _ptr(C), _ptr(H), prep.buf.data_ptr(), _ptr(n), _ptr(cj12), _ptr(ck12),
              N, nbf5, Q, nbeta, nalpha, S, _ptr(J_MO), _ptr(K_MO), _ptr(H_core), _ptr(elag), _ptr(Hmat), wp, wn,
              _stream(dev))
    return J_MO, K_MO, H_core, elag, Hmat
