"""Batched AMR blocks (bnsn_blocks_plan_create / bnsn_blocks_run): blocks of
uneven size with their own reactions, brem variant and quadrature order give
the same results as the per-configuration batched call on their points;
tuning picks a launch shape; a run captured in a CUDA graph replays to the
same results."""

import ctypes

import numpy as np
import pytest

import bns_nurates_gb300 as bn
from bns_nurates_gb300 import _capi as C

PARAMS = dict(brem_implementation=0)


def make_blocks(seed, nblocks, edges=(2, 3, 4, 5, 6, 8)):
    rng = np.random.default_rng(seed)
    blocks, first = [], 0
    for _ in range(nblocks):
        e = int(rng.choice(edges))
        count = e ** 3
        flags = (1, 1, 1, int(rng.integers(0, 2)), 1)
        brem = int(rng.integers(0, 3))
        nq = int(rng.choice((4, 6, 10)))
        blocks.append((first, count, flags, brem, nq))
        first += count
    return blocks, first


def test_blocks_plan_argument_errors(lib):
    """Bad block descriptors are rejected before any device work."""
    bad = (C.Block * 1)(C.Block(0, 10, bn.opacity_flags(), 0, 21))
    h = ctypes.c_void_p()
    rc = lib.bnsn_blocks_plan_create(bad, 1, ctypes.byref(bn.opacity_params()), 1, 0, 0, None,
                                     None, None, None, ctypes.byref(h))
    assert rc == C.ERR_NQUAD
    bad = (C.Block * 1)(C.Block(-1, 10, bn.opacity_flags(), 0, 4))
    rc = lib.bnsn_blocks_plan_create(bad, 1, ctypes.byref(bn.opacity_params()), 1, 0, 0, None,
                                     None, None, None, ctypes.byref(h))
    assert rc == C.ERR_ARG
    assert lib.bnsn_blocks_run(None, None, None, None, None) == C.ERR_ARG


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_blocks_match_direct_calls(cuda, precision):
    torch = cuda
    blocks, n = make_blocks(11, 40)
    eos_h, m1_h = bn.synthetic_points(20261203, n, first=5000)
    eos, m1 = torch.from_numpy(eos_h).cuda(), torch.from_numpy(m1_h).cuda()
    out = torch.full((20, n), float("nan"), dtype=torch.float64, device="cuda")
    plan = bn.BlocksPlan(blocks, eos, m1, out, precision=precision)
    plan.run(eos, m1, out)
    got = out.cpu().numpy()
    assert len(plan.groups()) >= 3
    for first, count, flags, brem, nq in blocks:
        sl = slice(first, first + count)
        e, m = eos[:, sl].contiguous(), m1[:, sl].contiguous()
        want = bn.m1_opacities(e, m, bn.opacity_flags(*flags),
                               bn.opacity_params(brem_implementation=brem),
                               bn.gauss_legendre(nq), precision=precision).cpu().numpy()
        # points are independent: same kernels, same arithmetic per point
        assert np.array_equal(got[:, sl], want), (first, count, flags, brem, nq)
    plan.close()


@pytest.mark.gpu
def test_blocks_tuning_and_graph_replay(cuda):
    torch = cuda
    blocks, n = make_blocks(12, 60, edges=(4, 6, 8, 10))
    eos_h, m1_h = bn.synthetic_points(7, n)
    eos, m1 = torch.from_numpy(eos_h).cuda(), torch.from_numpy(m1_h).cuda()
    out = torch.zeros((20, n), dtype=torch.float64, device="cuda")
    plan = bn.BlocksPlan(blocks, eos, m1, out, precision="mixed", tune=True)
    for g in plan.groups():
        assert g["chunk"] in (4096, 8192, 16384, 32768) or g["chunk"] == g["npts"]
        assert g["grid_scale"] in (2.0, 4.0)
    plan.run(eos, m1, out)
    torch.cuda.synchronize()
    ref = out.clone()
    out.zero_()
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.stream(s):
        plan.run(eos, m1, out, stream=s)   # warm-up on the capture stream
    torch.cuda.synchronize()
    out.zero_()
    with torch.cuda.graph(graph, stream=s):
        plan.run(eos, m1, out, stream=s)
    for _ in range(3):
        graph.replay()
    torch.cuda.synchronize()
    assert torch.equal(out, ref)
    plan.close()
