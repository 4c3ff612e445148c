"""ComplexF64 dense contractions on the FP64 tensor cores (QOB_OPT_FP64_TENSOR)
against the oracle.

With the context option on, dense operators (mul! -> BLAS zgemm,
src/operators_dense.jl:394-396) and the mode products of dense LazyTensor
factors (_tp_matmul_first!/_mid!/_last!, src/operators_lazytensor.jl:281-428)
whose contracted dimension is at least 64, applied to at least 8 kets, run as
DMMA (mma.sync m8n8k4 f64) tiles; fewer kets stay on the FMA kernels.  Checked
at the ComplexF64 bar (relative l2 < 1e-12) against the oracle: a 700 x 500
dense operator on kets from the left and on the rows of an operator from the
right (1 ket: the FMA path under the option; 9: a ragged ket tile; 16), and
mode products with the factor on the first, a middle and the last subsystem,
on 1, 11 and 16 kets, with a complex beta.
"""
import numpy as np
import pytest

import qobgpu as Q
from helpers import rand_op
from qobgpu import operators as O
from test_gpu_parity import check

pytestmark = pytest.mark.gpu

TOL64 = 1e-12
AL = 0.7 - 0.2j
BE = 0.4 - 0.9j


@pytest.fixture
def fp64_tensor():
    from qobgpu import _lib as L
    from qobgpu.device import get_context, raise_for

    ctx = get_context(0)
    raise_for(L.lib().qob_set_option(ctx.ptr, L.QOB_OPT_FP64_TENSOR, 1), ctx)
    yield
    raise_for(L.lib().qob_set_option(ctx.ptr, L.QOB_OPT_FP64_TENSOR, 0), ctx)


@pytest.mark.parametrize("ncols", [1, 9, 16])
def test_dmma_dense_operator(fp64_tensor, ncols):
    rng = Q.Rng(180 + ncols)
    bl, br = Q.GenericBasis(700), Q.GenericBasis(500)
    D = rand_op(rng, bl, br)
    X = O.Operator(br, Q.GenericBasis(ncols), rng.kets_data(500, ncols))
    Y = O.Operator(bl, Q.GenericBasis(ncols), rng.kets_data(700, ncols))
    check(Y, D, X, AL, BE, TOL64)
    check(Y, D, X, AL, 0.0, TOL64)
    R = O.Operator(Q.GenericBasis(ncols), bl, np.asfortranarray(rng.complex_normal(ncols * 700).reshape(ncols, 700, order="F")))
    Z = O.Operator(Q.GenericBasis(ncols), br, np.asfortranarray(rng.complex_normal(ncols * 500).reshape(ncols, 500, order="F")))
    check(Z, R, D, AL, BE, TOL64)


def _dense_factor(rng, d):
    return O.Operator(Q.GenericBasis(d), Q.GenericBasis(d), np.asfortranarray(rng.complex_normal(d * d).reshape(d, d, order="F")))


@pytest.mark.parametrize("ncols", [1, 11, 16])
@pytest.mark.parametrize("dims,sites", [((80, 3, 70), (1, 3)), ((5, 96, 7), (2,)), ((9, 72), (2,)), ((66, 4), (1,))])
def test_dmma_mode_products(fp64_tensor, dims, sites, ncols):
    rng = Q.Rng(190 + len(dims) + ncols)
    b = Q.tensor_basis(*[Q.GenericBasis(d) for d in dims])
    facs = tuple(_dense_factor(rng, dims[s - 1]) for s in sites)
    op = O.LazyTensor(b, b, sites, facs, 0.3 - 0.1j)
    n = len(b)
    X = O.Operator(b, Q.GenericBasis(ncols), rng.kets_data(n, ncols))
    Y = O.Operator(b, Q.GenericBasis(ncols), rng.kets_data(n, ncols))
    check(Y, op, X, AL, BE, TOL64)
    if ncols == 1:
        psi, out = Q.Ket(b, rng.ket_data(n)), Q.Ket(b, rng.ket_data(n))
        check(out, op, psi, AL, BE, TOL64)
