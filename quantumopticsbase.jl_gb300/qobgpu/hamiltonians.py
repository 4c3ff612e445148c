"""The benchmark Hamiltonians, built the way a user of the reference would.

Each is an explicit ``LazySum(factors, (LazyTensor, ...))`` so the term counts
stay as written: ``+`` on two single-factor LazyTensors with the same indices
would merge them (src/operators_lazytensor.jl:100-114).

* ``jaynes_cummings``  -- FockBasis(N1) ⊗ SpinBasis(1/2) ⊗ FockBasis(N2), 7 terms:
  ω n₁, ω n₃, (Δ/2) σz₂, g a₁†σ₋, g a₁σ₊, g σ₋a₃†, g σ₊a₃; ω, Δ, g ~ U(0.5, 2).
* ``heisenberg_chain`` -- open spin-1/2 chain, J(σxσx + σyσy + σzσz) on every bond
  plus h_i σz_i with h_i ~ U(-1, 1): 3(n-1) + n terms (53 at 14 spins).
* ``two_mode_cavity``  -- FockBasis(n1) ⊗ FockBasis(n2), 4 terms:
  ω₁n₁, ω₂n₂, χ n₁n₂, ε(a₁ + a₁†); parameters ~ U(0.1, 2).
"""
from __future__ import annotations

import numpy as np

from .bases import FockBasis, SpinBasis, tensor
from .operators import (LazySum, LazyTensor, Operator, add, create, destroy, number, sigmam, sigmap,
                        sigmax, sigmay, sigmaz, sparse)
from .rng import Rng


def jaynes_cummings(N1: int = 15, N2: int = 15, seed: int = 1, dtype=np.complex128) -> LazySum:
    rng = Rng(seed)
    omega, delta, g = rng.uniform(3, 0.5, 2.0)
    bf1, bs, bf2 = FockBasis(N1), SpinBasis("1/2"), FockBasis(N2)
    b = tensor(bf1, bs, bf2)
    terms = [
        (omega, LazyTensor(b, b, (1,), (number(bf1, dtype),))),
        (omega, LazyTensor(b, b, (3,), (number(bf2, dtype),))),
        (delta / 2, LazyTensor(b, b, (2,), (sigmaz(bs, dtype),))),
        (g, LazyTensor(b, b, (1, 2), (create(bf1, dtype), sigmam(bs, dtype)))),
        (g, LazyTensor(b, b, (1, 2), (destroy(bf1, dtype), sigmap(bs, dtype)))),
        (g, LazyTensor(b, b, (2, 3), (sigmam(bs, dtype), create(bf2, dtype)))),
        (g, LazyTensor(b, b, (2, 3), (sigmap(bs, dtype), destroy(bf2, dtype)))),
    ]
    return LazySum(b, b, [c for c, _ in terms], tuple(t for _, t in terms))


def heisenberg_chain(nspins: int = 14, J: float = 1.0, seed: int = 1, dtype=np.complex128) -> LazySum:
    rng = Rng(seed)
    h = rng.uniform(nspins, -1.0, 1.0)
    bs = SpinBasis("1/2")
    b = tensor(*([bs] * nspins))
    sx, sy, sz = sigmax(bs, dtype), sigmay(bs, dtype), sigmaz(bs, dtype)
    factors, ops = [], []
    for i in range(1, nspins):
        for s in (sx, sy, sz):
            factors.append(J)
            ops.append(LazyTensor(b, b, (i, i + 1), (s, s)))
    for i in range(1, nspins + 1):
        factors.append(h[i - 1])
        ops.append(LazyTensor(b, b, (i,), (sz,)))
    return LazySum(b, b, factors, tuple(ops))


def two_mode_cavity(n1: int, n2: int, seed: int = 1, dtype=np.complex128) -> LazySum:
    rng = Rng(seed)
    w1, w2, chi, eps = rng.uniform(4, 0.1, 2.0)
    b1, b2 = FockBasis(n1), FockBasis(n2)
    b = tensor(b1, b2)
    drive = add(destroy(b1, dtype), create(b1, dtype))
    ops = (
        LazyTensor(b, b, (1,), (number(b1, dtype),)),
        LazyTensor(b, b, (2,), (number(b2, dtype),)),
        LazyTensor(b, b, (1, 2), (number(b1, dtype), number(b2, dtype))),
        LazyTensor(b, b, (1,), (drive,)),
    )
    return LazySum(b, b, [w1, w2, chi, eps], ops)


def jaynes_cummings_sparse(N1: int = 31, N2: int = 63, seed: int = 1, dtype=np.complex128) -> Operator:
    """``sparse(H)`` of the Jaynes-Cummings LazySum (src/operators_lazysum.jl:81)."""
    H = sparse(jaynes_cummings(N1, N2, seed, dtype))
    if dtype == np.complex64:
        H = Operator(H.basis_l, H.basis_r, H.data.astype(np.complex64))
    return H


def random_density_columns(dim: int, ncols: int, rank: int = 64, seed: int = 2,
                           dtype=np.complex128) -> np.ndarray:
    """First ``ncols`` columns of a random dim x dim density matrix (PSD, trace 1),
    built as A A† / tr(A A†) with A a complex-Gaussian dim x rank matrix."""
    rng = Rng(seed)
    A = rng.complex_normal(dim * rank).reshape(dim, rank, order="F")
    tr = np.sum(np.abs(A) ** 2)
    rho = (A @ A[:ncols, :].conj().T) / tr
    return np.asfortranarray(rho.astype(dtype))
