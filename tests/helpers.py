"""Shared builders and metrics for the parity tests (oracle vs libqobgpu)."""
from __future__ import annotations

import numpy as np

import oracle as OR
import qobgpu as Q
from qobgpu import operators as O


def rel_l2(a, b) -> float:
    a = np.asarray(a)
    b = np.asarray(b)
    d = np.linalg.norm((a - b).ravel())
    n = np.linalg.norm(b.ravel())
    return float(d / n) if n > 0 else float(d)


def rand_op(rng: Q.Rng, bl, br, dtype=np.complex128, density=None) -> O.Operator:
    """Random dense operator (the reference's randoperator, with the project's generator)."""
    m, n = len(bl), len(br)
    a = rng.complex_normal(m * n).reshape(m, n, order="F").astype(dtype)
    if density is not None:
        mask = rng.uniform(m * n).reshape(m, n, order="F") < density
        a = np.where(mask, a, 0)
    return O.Operator(bl, br, np.asfortranarray(a))


def rand_state(rng: Q.Rng, b, kind=Q.Ket, dtype=np.complex128):
    return kind(b, rng.ket_data(len(b), dtype))


def dense_of(op) -> np.ndarray:
    return np.asarray(O.dense(op).data)


def host_copy(x):
    """numpy copy of a state's / operator's data."""
    d = x.data
    if hasattr(d, "cpu"):
        return d.cpu().numpy()
    return np.array(O._to_dense_array(d) if isinstance(x, O.Operator) else d, copy=True)
