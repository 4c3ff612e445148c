"""Generates tests/golden/golden.npz: inputs and expected outputs of mul! cases.

The reference's test suite stores no vectors (its tests compare lazy operators
with their dense materialisation, test/test_operators_lazytensor.jl:237-496,
test/test_operators_lazysum.jl:255-347).  These fixtures re-create those cases
on seeded inputs and record the expected results computed the way those tests
compute them: the operator materialised densely (kron in the reference's
first-subsystem-fastest order, src/operators_dense.jl:134) and applied with
numpy -- independently of both the oracle and the GPU library.

Run from the repository root:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "quantumopticsbase.jl_gb300"))

import qobgpu as Q  # noqa: E402
from qobgpu import operators as O  # noqa: E402
from qobgpu.hamiltonians import heisenberg_chain, jaynes_cummings, jaynes_cummings_sparse, two_mode_cavity  # noqa: E402

ALPHA, BETA = 0.7 - 0.2j, 0.3


def rand_op(rng, bl, br, density=None):
    m, n = len(bl), len(br)
    a = rng.complex_normal(m * n).reshape(m, n, order="F")
    if density is not None:
        a = np.where(rng.uniform(m * n).reshape(m, n, order="F") < density, a, 0)
    return O.Operator(bl, br, np.asfortranarray(a))


def iso_lazytensor():
    bl = Q.tensor_basis(Q.FockBasis(2), Q.GenericBasis(2), Q.SpinBasis("1/2"), Q.GenericBasis(1), Q.GenericBasis(2))
    br = Q.tensor_basis(Q.FockBasis(2), Q.GenericBasis(2), Q.SpinBasis("1/2"), Q.GenericBasis(2), Q.GenericBasis(1))
    return O.LazyTensor(bl, br, (1, 3), (O.number(bl.bases[0]), O.sigmax(bl.bases[2])))


def mixed_lazytensor():
    rng = Q.Rng(501)
    b1a, b1b, b2a, b2b, b3a, b3b = (Q.GenericBasis(k) for k in (2, 3, 1, 4, 6, 5))
    bl, br = Q.tensor_basis(b1a, b2a, b3a), Q.tensor_basis(b1b, b2b, b3b)
    facs = (rand_op(rng, b1a, b1b), O.dagger(rand_op(rng, b2b, b2a)), O.sparse(rand_op(rng, b3a, b3b)))
    return O.LazyTensor(bl, br, (1, 2, 3), facs, 0.1)


def lazyproduct():
    rng = Q.Rng(502)
    bs = [Q.GenericBasis(k) for k in (3, 5, 4, 6)]
    return O.LazyProduct(tuple(rand_op(rng, bs[i], bs[i + 1]) for i in range(3)), factor=0.5 - 0.1j)


def sparse_small():
    rng = Q.Rng(503)
    b = Q.GenericBasis(60)
    return O.sparse(rand_op(rng, b, b, density=0.3))


# name -> (builder, form); form: "ket" (H psi), "bra" (psi H), "opL" (H rho), "opR" (rho H)
CASES = {
    "jc_3_3_ket": (lambda: jaynes_cummings(3, 3, seed=1), "ket"),
    "jc_15_15_ket": (lambda: jaynes_cummings(15, 15, seed=1), "ket"),
    "heisenberg6_ket": (lambda: heisenberg_chain(6, seed=3), "ket"),
    "heisenberg6_bra": (lambda: heisenberg_chain(6, seed=3), "bra"),
    "heisenberg5_opL": (lambda: heisenberg_chain(5, seed=4), "opL"),
    "heisenberg5_opR": (lambda: heisenberg_chain(5, seed=4), "opR"),
    "cavity_4_6_ket": (lambda: two_mode_cavity(4, 6, seed=10), "ket"),
    "jc_sparse_7_7_ket": (lambda: jaynes_cummings_sparse(7, 7, seed=1), "ket"),
    "isometry_opL": (iso_lazytensor, "opL"),
    "mixed_lazytensor_ket": (mixed_lazytensor, "ket"),
    "mixed_lazytensor_bra": (mixed_lazytensor, "bra"),
    "lazyproduct_ket": (lazyproduct, "ket"),
    "sparse60_opL": (sparse_small, "opL"),
    "sparse60_opR": (sparse_small, "opR"),
}


def make_inputs(H, form, seed):
    rng = Q.Rng(seed)
    m, n = len(H.basis_l), len(H.basis_r)
    if form == "ket":
        return rng.complex_normal(n), rng.complex_normal(m)
    if form == "bra":
        return rng.complex_normal(m), rng.complex_normal(n)
    k = 7
    if form == "opL":
        return (rng.complex_normal(n * k).reshape(n, k, order="F"), rng.complex_normal(m * k).reshape(m, k, order="F"))
    return (rng.complex_normal(k * m).reshape(k, m, order="F"), rng.complex_normal(k * n).reshape(k, n, order="F"))


def expected(H, form, x, y):
    D = np.asarray(O.dense(H).data)
    if form in ("ket", "opL"):
        return ALPHA * (D @ x) + BETA * y
    return ALPHA * (x @ D) + BETA * y


def main():
    out = {}
    for i, (name, (build, form)) in enumerate(sorted(CASES.items())):
        H = build()
        x, y = make_inputs(H, form, 900 + i)
        out[name + "__x"] = np.asarray(x, np.complex128)
        out[name + "__y"] = np.asarray(y, np.complex128)
        out[name + "__expected"] = expected(H, form, x, y)
    np.savez_compressed(os.path.join(HERE, "golden.npz"), alpha=ALPHA, beta=BETA, **out)
    print(f"wrote {len(CASES)} cases")


if __name__ == "__main__":
    main()
