"""Seeded synthetic inputs for the RI / full-ERI JK path.

PyNOF obtains ``b_mnl`` from psi4 (``pynof/integrals.py:33-49``: 3-centre ERIs
contracted with the fitting metric to the power -1/2) and ``C``/``H`` from the
molecule.  psi4 is not part of this project, so every workload here is
synthetic, drawn with numpy's ``Generator(PCG64(seed))`` in a fixed order
(b, C, H, n):

* ``b[m, n, Q]``: standard normal scaled by ``exp(-0.05 (m + n))``, then
  symmetrised in (m, n) -- the same symmetry real 3-index factors carry;
* ``C``: the Q factor of a QR decomposition of a standard normal N x N matrix
  (an orthogonal MO coefficient matrix);
* ``H``: ``0.5 (A + A^T)`` of a standard normal N x N matrix;
* ``n``: uniform(0, 1) occupations of the nbf5 natural orbitals, sorted
  descending.

The PNOF orbital structure (closed shell, no inactive orbitals, softmax
occupations, GNOF = PNOF8) is described by :class:`Structure`, which carries the
subset of ``pynof.param`` attributes (``pynof/parameters.py:17-112``) that the
hot path reads.
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np


@dataclasses.dataclass
class Structure:
    """Orbital-space sizes of one NOF problem (mirrors ``pynof.param``)."""

    nbf: int
    nbfaux: int
    ndoc: int
    ncwo: int
    no1: int = 0
    nsoc: int = 0
    MSpin: int = 0
    HighSpin: bool = False
    RI: bool = True
    gpu: bool = True
    jit: bool = False
    ipnof: int = 8
    occ_method: str = "Softmax"

    def __post_init__(self):
        self.nbeta = self.no1 + self.ndoc
        self.nalpha = self.nbeta + self.nsoc
        self.ndns = self.ndoc + self.nsoc
        self.nac = self.ndoc * (1 + self.ncwo)
        self.nbf5 = self.no1 + self.nac + self.nsoc
        if self.nbf5 > self.nbf:
            raise ValueError(f"nbf5={self.nbf5} exceeds nbf={self.nbf}")
        self.no0 = self.nbf - self.nbf5
        self.noptorb = self.nbf
        self.nv = self.ncwo * self.ndoc
        self.nvar = self.nbf * (self.nbf - 1) // 2 - self.no0 * (self.no0 - 1) // 2
        self.maxloop = 30
        self.alpha = 0.02

    @classmethod
    def for_nbf(cls, nbf: int, naux: int | None = None, ncwo: int = 4) -> "Structure":
        """Sizes used for the batched / served workloads: ndoc = nbf // 10,
        nbf5 = ndoc (1 + ncwo) (about nbf / 2), naux = 4 nbf."""
        ndoc = max(1, nbf // 10)
        return cls(nbf=nbf, nbfaux=naux if naux is not None else 4 * nbf, ndoc=ndoc, ncwo=ncwo)


#: Named workloads.  ``c1`` is the water/cc-pVDZ shape, ``c2`` the medium
#: FP64 case, ``c3`` the nbf=600 case the JK-build throughput is quoted on.
WORKLOADS = {
    "c1": dict(nbf=24, nbfaux=116, ndoc=4, ncwo=5),
    "water": dict(nbf=24, nbfaux=116, ndoc=5, ncwo=3),
    "ragged": dict(nbf=37, nbfaux=150, ndoc=4, ncwo=4),
    "c2": dict(nbf=300, nbfaux=1200, ndoc=30, ncwo=4),
    "c3": dict(nbf=600, nbfaux=2400, ndoc=60, ncwo=4),
}


def structure(name: str) -> Structure:
    return Structure(**WORKLOADS[name])


def make_inputs(st: Structure, seed: int = 0):
    """Draw (b, C, H, n) for ``st`` in the fixed order b, C, H, n."""
    N, Q, P = st.nbf, st.nbfaux, st.nbf5
    rng = np.random.Generator(np.random.PCG64(seed))
    b = rng.standard_normal((N, N, Q))
    idx = np.arange(N, dtype=np.float64)
    b *= np.exp(-0.05 * (idx[:, None] + idx[None, :]))[:, :, None]
    b += b.transpose(1, 0, 2).copy()
    b *= 0.5
    C, _ = np.linalg.qr(rng.standard_normal((N, N)))
    C = np.ascontiguousarray(C)
    A = rng.standard_normal((N, N))
    H = 0.5 * (A + A.T)
    n = np.sort(rng.uniform(0.0, 1.0, P))[::-1].copy()
    return b, C, H, n


def batch_sizes(count: int, lo: int = 24, hi: int = 400, seed: int = 7) -> list[int]:
    """nbf drawn log-uniform in [lo, hi] (batched / served workloads)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    u = rng.uniform(math.log(lo), math.log(hi), count)
    return [int(round(math.exp(x))) for x in u]
