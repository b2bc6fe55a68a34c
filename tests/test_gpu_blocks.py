"""Batched AMR blocks (bnsn_blocks_plan_create / bnsn_blocks_run): blocks of
uneven size with their own reactions, brem variant and quadrature order give
the same results as the per-configuration batched call on their points;
tuning picks a launch shape; a run captured in a CUDA graph replays to the
same results; a run is one launch per phase kernel and step for all groups, and
a scratch limit that splits the points into many steps changes no result."""

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


def test_blocks_options_and_layout_argument_errors(lib):
    """bnsn_blocks_set_options rejects negative values and keeps the last
    valid options; bnsn_blocks_plan_layout rejects a NULL plan (no device
    work in either)."""
    assert lib.bnsn_blocks_set_options(-1, 0) == C.ERR_ARG
    assert lib.bnsn_blocks_set_options(0, -5) == C.ERR_ARG
    assert lib.bnsn_blocks_set_options(1 << 30, 4096) == C.OK
    assert lib.bnsn_blocks_set_options(0, 0) == C.OK
    steps = ctypes.c_int(-7)
    assert lib.bnsn_blocks_plan_layout(None, ctypes.byref(steps), None, None) == C.ERR_ARG
    assert steps.value == -7
    assert lib.bnsn_blocks_plan_groups(None) == 0


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
        # points are independent: the same arithmetic per point.  The plan
        # runs the multi-group instantiations of the phase kernels, which the
        # compiler may contract differently (a*b + c fused or not): the FP64
        # path is bitwise equal, the mixed path's FP64 passes over flagged
        # points may differ in the last bits
        if precision == "fp64":
            assert np.array_equal(got[:, sl], want), (first, count, flags, brem, nq)
        else:
            np.testing.assert_allclose(got[:, sl], want, rtol=1e-13, atol=0,
                                       err_msg=str((first, count, flags, brem, nq)))
    plan.close()


@pytest.mark.gpu
def test_blocks_tuning_and_graph_replay(cuda):
    torch = cuda
    blocks, n = make_blocks(12, 60, edges=(4, 6, 8, 10))
    eos_h, m1_h = bn.synthetic_points(7, n)
    eos, m1 = torch.from_numpy(eos_h).cuda(), torch.from_numpy(m1_h).cuda()
    out = torch.zeros((20, n), dtype=torch.float64, device="cuda")
    plan = bn.BlocksPlan(blocks, eos, m1, out, precision="mixed", tune=True)
    lay = plan.layout()
    assert lay["steps"] >= 2 and lay["steps"] % 2 == 0
    for g in plan.groups():
        # every group's points spread evenly over the steps
        assert g["chunk"] == -(-g["npts"] // lay["steps"])
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


def expected_launches(groups, steps):
    """Kernel launches of a mixed run: the descriptor update, then per step the
    phases of the union of the groups with points in the step -- point,
    prelude, pair, brem per variant, NES fast and the two flagged NES passes,
    final, and the FP64 pair and brem passes with a second final."""
    n = 1
    for s in range(steps):
        live = [g for g in groups if s * g["chunk"] < g["npts"]]
        pair = any(g["reactions"] & 2 for g in live)
        brems = len({g["brem"] for g in live if g["reactions"] & 4})
        nes = any(g["reactions"] & 8 for g in live)
        n += 3 + pair + brems + 3 * nes
        if pair or brems:
            n += pair + brems + 1
    return n


@pytest.mark.gpu
def test_blocks_one_launch_per_phase_and_steps(cuda):
    """Each step launches every phase kernel once for all groups (grid z), and
    other step layouts (a small scratch limit, small steps, one step per
    stream) give the same results bit for bit."""
    torch = cuda
    lib = C.load()
    blocks, n = make_blocks(13, 50, edges=(3, 4, 6, 8))
    eos_h, m1_h = bn.synthetic_points(99, n, first=1000)
    eos, m1 = torch.from_numpy(eos_h).cuda(), torch.from_numpy(m1_h).cuda()
    outs = []
    try:
        # (scratch limit, points per step): default, scratch-limited, small
        # steps, one step per stream
        for limit, step in ((0, 0), (64 * 6400, 0), (0, 700), (0, 10 ** 9)):
            bn.BlocksPlan.set_options(limit, step)
            out = torch.full((20, n), float("nan"), dtype=torch.float64, device="cuda")
            plan = bn.BlocksPlan(blocks, eos, m1, out, precision="mixed")
            lay = plan.layout()
            if limit:
                assert lay["scratch_bytes"] <= max(limit, 2 * len(plan.groups()) * 6400)
            if step:
                assert lay["steps"] >= max(2, n // step)
            if step == 10 ** 9:
                assert lay["steps"] == 2
            torch.cuda.synchronize()
            k0 = lib.bnsn_kernel_launches()
            plan.run(eos, m1, out)
            torch.cuda.synchronize()
            launches = lib.bnsn_kernel_launches() - k0
            assert launches == expected_launches(plan.groups(), lay["steps"]), (launches, lay)
            outs.append(out.cpu())
            plan.close()
        assert outs[1].isfinite().all()
        for o in outs[1:]:
            assert torch.equal(outs[0], o)
    finally:
        bn.BlocksPlan.set_options()
