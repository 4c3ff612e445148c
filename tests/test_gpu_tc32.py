"""ComplexF32 dense operators on the 5th-generation tensor cores
(QOB_OPT_FP32_TENSOR: tcgen05.mma kind::tf32, accumulator in tensor memory,
operand tiles loaded by TMA, each operand split into a TF32 head and tail)
against the oracle (the reference's dense mul!, src/operators_dense.jl:394-396,
restated in FP64), at the ComplexF32 tolerance 1e-5 (relative l2): kets from
the left in every tile width the kernel has (1 .. 100 kets: 16, 32 and 64 kets
per pass), rows of an operator from the right, beta = 0 over a NaN-filled
output, a matrix whose sides are not multiples of the tile sizes, the
4096 x 4096 operator on 16 kets (row tiles split over several blocks, partial
products added in order) and a 19,500 x 64 operator (more row tiles than one
wave of blocks: every block writes whole row tiles); and the mode products of
dense LazyTensor factors of 64 or more (the reference's _tp_matmul_first! /
_mid! / _last!, src/operators_lazytensor.jl:281-428) with the factor on the
first, a middle and the last subsystem, on 1, 16 and 100 kets, from the left
and on the rows of an operator from the right; the device status word stays
clear.
"""
import ctypes as C

import numpy as np
import pytest

import qobgpu as Q
from helpers import rand_op
from qobgpu import operators as O
from test_gpu_parity import check

pytestmark = pytest.mark.gpu

TOL32 = 1e-5
AL = 0.7 - 0.2j
BE = 0.4 - 0.9j


@pytest.fixture
def fp32_tensor():
    from qobgpu import _lib as L
    from qobgpu.device import get_context, raise_for

    ctx = get_context(0)
    raise_for(L.lib().qob_set_option(ctx.ptr, L.QOB_OPT_FP32_TENSOR, 1), ctx)
    yield
    raise_for(L.lib().qob_set_option(ctx.ptr, L.QOB_OPT_FP32_TENSOR, 0), ctx)
    flags = C.c_uint()
    raise_for(L.lib().qob_device_status(ctx.ptr, None, C.byref(flags)), ctx)
    assert flags.value == 0


@pytest.mark.parametrize("ncols", [1, 3, 16, 17, 40, 64, 100])
def test_tc32_dense_left(fp32_tensor, ncols):
    rng = Q.Rng(300 + ncols)
    bl, br = Q.GenericBasis(700), Q.GenericBasis(500)
    D = rand_op(rng, bl, br)
    X = O.Operator(br, Q.GenericBasis(ncols), rng.kets_data(500, ncols))
    Y = O.Operator(bl, Q.GenericBasis(ncols), rng.kets_data(700, ncols))
    check(Y, D, X, AL, BE, TOL32, np.complex64)
    Yn = O.Operator(bl, Q.GenericBasis(ncols), np.full((700, ncols), np.nan, np.complex128, order="F"))
    check(Yn, D, X, AL, 0.0, TOL32, np.complex64)


def test_tc32_dense_right_and_odd_sizes(fp32_tensor):
    rng = Q.Rng(320)
    bl, br = Q.GenericBasis(333), Q.GenericBasis(257)
    D = rand_op(rng, bl, br)
    R = O.Operator(Q.GenericBasis(5), bl, np.asfortranarray(rng.complex_normal(5 * 333).reshape(5, 333, order="F")))
    Z = O.Operator(Q.GenericBasis(5), br, np.asfortranarray(rng.complex_normal(5 * 257).reshape(5, 257, order="F")))
    check(Z, R, D, AL, BE, TOL32, np.complex64)
    X = O.Operator(br, Q.GenericBasis(7), rng.kets_data(257, 7))
    Y = O.Operator(bl, Q.GenericBasis(7), rng.kets_data(333, 7))
    check(Y, D, X, AL, BE, TOL32, np.complex64)


def test_tc32_dense_4096_on_16_kets(fp32_tensor):
    rng = Q.Rng(330)
    b = Q.GenericBasis(4096)
    D = rand_op(rng, b, b)
    X = O.Operator(b, Q.GenericBasis(16), rng.kets_data(4096, 16))
    Y = O.Operator(b, Q.GenericBasis(16), rng.kets_data(4096, 16))
    check(Y, D, X, AL, BE, TOL32, np.complex64)


def test_tc32_dense_tall_whole_row_tiles(fp32_tensor):
    # 305 row tiles of 64 rows: at least one wave of blocks, so each block takes
    # whole row tiles (its full k range) and writes y itself, with no reduction
    rng = Q.Rng(340)
    bl, br = Q.GenericBasis(19500), Q.GenericBasis(64)
    D = rand_op(rng, bl, br)
    X = O.Operator(br, Q.GenericBasis(3), rng.kets_data(64, 3))
    Y = O.Operator(bl, Q.GenericBasis(3), rng.kets_data(19500, 3))
    check(Y, D, X, AL, BE, TOL32, np.complex64)


def _dense_factor(rng, d):
    return O.Operator(Q.GenericBasis(d), Q.GenericBasis(d),
                      np.asfortranarray(rng.complex_normal(d * d).reshape(d, d, order="F")))


@pytest.mark.parametrize("dims,sites,ncols", [(d, s, c) for d, s in (((80, 3, 70), (1, 3)), ((5, 96, 7), (2,)),
                                                                       ((9, 72), (2,)), ((66, 4), (1,)))
                                               for c in (1, 16, 100)] + [((200, 3, 200), (1, 3), 16)])
def test_tc32_mode_products(fp32_tensor, dims, sites, ncols):
    rng = Q.Rng(360 + len(dims) + ncols + dims[0])
    b = Q.tensor_basis(*[Q.GenericBasis(d) for d in dims])
    facs = tuple(_dense_factor(rng, dims[s - 1]) for s in sites)
    op = O.LazyTensor(b, b, sites, facs, 0.3 - 0.1j)
    n = len(b)
    X = O.Operator(b, Q.GenericBasis(ncols), rng.kets_data(n, ncols))
    Y = O.Operator(b, Q.GenericBasis(ncols), rng.kets_data(n, ncols))
    check(Y, op, X, AL, BE, TOL32, np.complex64)
    if ncols == 16 and len(dims) == 3 and dims[0] < 100:
        R = O.Operator(Q.GenericBasis(5), b, np.asfortranarray(rng.complex_normal(5 * n).reshape(5, n, order="F")))
        Z = O.Operator(Q.GenericBasis(5), b, np.asfortranarray(rng.complex_normal(5 * n).reshape(5, n, order="F")))
        check(Z, R, op, AL, BE, TOL32, np.complex64)


@pytest.mark.parametrize("which,k", [("dense", 16), ("dense", 7), ("mode_products", 16)])
def test_tc32_pdl_keeps_chained_applications_ordered(fp32_tensor, which, k):
    """QOB_OPT_PDL on the tensor-core path: the split, GEMM and reduce kernels
    of each application are launched with programmatic dependent launch (the
    GEMM's set-up overlaps the split, every kernel waits for its predecessor
    before touching memory).  A chain y1 = A x, y2 = A y1, y3 = A y2 of
    ComplexF32 applications recorded into a CUDA graph and replayed equals the
    oracle's chain at the ComplexF32 tolerance and is bitwise equal to the same
    chain without PDL; a dense 1024 x 1024 operator on 16 kets (row tiles split
    over several blocks, partial products reduced), the same on 7 kets (a
    ragged column tile: the split's buffers are cleared by a memset that the
    split launch follows) and two 200 x 200 mode products on a 200 x 3 x 200
    basis (two split -> GEMM -> reduce chains per application)."""
    import torch

    import oracle as OR
    from helpers import rel_l2
    from qobgpu import _lib as L
    from qobgpu.device import dtype_code, get_context, handle, raise_for

    rng = Q.Rng(380)
    if which == "dense":
        b = Q.GenericBasis(1024)
        op = rand_op(rng, b, b)
        alpha = 1.0 / 32.0
    else:
        b = Q.tensor_basis(Q.GenericBasis(200), Q.GenericBasis(3), Q.GenericBasis(200))
        op = O.LazyTensor(b, b, (1, 3), (_dense_factor(rng, 200), _dense_factor(rng, 200)), 1.0)
        alpha = 1.0 / 200.0
    n = len(b)
    X = rng.kets_data(n, k)
    node = OR.build_node(op)
    ref = [np.asfortranarray(X.astype(np.complex64).astype(np.complex128))]
    for _ in range(3):
        r = np.zeros_like(ref[-1])
        OR.mul_kets_threaded(node, alpha, np.asfortranarray(ref[-1]), 0.0, r, 8)
        ref.append(r)
    lib = L.lib()
    ctx = get_context(0)
    hd = handle(ctx, op)
    code = dtype_code(np.complex64)
    stream = torch.cuda.Stream()
    sp = C.c_void_p(stream.cuda_stream)
    outs = {}
    try:
        for pdl in (0, 1):
            raise_for(lib.qob_set_option(ctx.ptr, L.QOB_OPT_PDL, pdl), ctx)
            bufs = [torch.as_tensor(np.ascontiguousarray(X.T), device="cuda:0").to(torch.complex64).t()]
            bufs += [torch.zeros(k, n, dtype=torch.complex64, device="cuda:0").t() for _ in range(3)]

            def chain():
                for i in range(3):
                    raise_for(lib.qob_mul(ctx.ptr, L.QOB_LEFT, 0, hd.ptr, code, alpha, 0.0,
                                          C.c_void_p(bufs[i].data_ptr()), n, k, n, 0.0, 0.0,
                                          C.c_void_p(bufs[i + 1].data_ptr()), n, k, n, sp), ctx)

            torch.cuda.synchronize()
            chain()  # direct launches (builds the tiled matrix on first use)
            stream.synchronize()
            g = C.c_void_p()
            raise_for(lib.qob_graph_begin(ctx.ptr, sp), ctx)
            chain()
            raise_for(lib.qob_graph_end(ctx.ptr, sp, C.byref(g)), ctx)
            for t in bufs[1:]:
                t.zero_()
            torch.cuda.synchronize()
            for _ in range(3):
                raise_for(lib.qob_graph_launch(ctx.ptr, g, sp), ctx)
            stream.synchronize()
            lib.qob_graph_free(ctx.ptr, g)
            outs[pdl] = [t.cpu().numpy().astype(np.complex128) for t in bufs[1:]]
    finally:
        raise_for(lib.qob_set_option(ctx.ptr, L.QOB_OPT_PDL, 0), ctx)
    for i in range(3):
        assert rel_l2(outs[1][i], ref[i + 1]) < TOL32, (i, rel_l2(outs[1][i], ref[i + 1]))
        assert np.array_equal(outs[1][i], outs[0][i])
