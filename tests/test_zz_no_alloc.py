"""bnsn_m1_opacities_noalloc: grey opacities with scratch in a static device
array, for callers whose device memory belongs to their own allocator and
that therefore cannot let the library allocate.  Called through the C ABI and
compared with bnsn_m1_opacities.

Collected last (file name) so it also runs after every other GPU test has
used the library in the same process; one case runs it as the first library
call of a fresh process.
"""

import ctypes
import os
import subprocess
import sys
import textwrap

import numpy as np
import pytest

TOL = 1e-12
REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _call(entry, eos, m1, flags, params, q, out, n, stream, precision=0):
    from bns_nurates_gb300 import api
    E, M, O = api._eos_soa(eos), api._m1_soa(m1), api._grey_soa(out)
    return entry(ctypes.byref(q), ctypes.byref(q), ctypes.byref(flags), ctypes.byref(params),
                 ctypes.byref(E), ctypes.byref(M), None, 1, precision, ctypes.byref(O), n,
                 stream)


def _assert_close(g, want_h):
    assert np.all(np.isfinite(g) == np.isfinite(want_h))
    both = np.isfinite(g) & np.isfinite(want_h)
    d = np.abs(g - want_h)[both]
    scale = np.abs(want_h)[both]
    assert np.all(d <= TOL * scale), float(np.max(d / np.where(scale > 0, scale, 1)))


def test_noalloc_rejects_too_many_points(lib):
    """npts above the static capacity fails with BNSN_ERR_ARG before any device work."""
    import bns_nurates_gb300 as bn
    from bns_nurates_gb300 import _capi as C
    n = C.NOALLOC_MAX_POINTS + 1
    eos, m1 = bn.synthetic_points(7, n)
    out = np.empty((20, n))
    rc = _call(C.load().bnsn_m1_opacities_noalloc, eos, m1, bn.opacity_flags(),
               bn.opacity_params(), bn.gauss_legendre(4), out, n, None)
    assert rc == C.ERR_ARG
    msg = C.load().bnsn_last_error().decode()
    assert "BNSN_NOALLOC_MAX_POINTS" in msg and "4096" in msg


@pytest.mark.gpu
@pytest.mark.parametrize("flags,brem,nq,n", [
    ((1, 1, 1, 1, 1), 0, 10, 4096),   # all reactions, HR98, the full static capacity
    ((1, 1, 1, 1, 1), 2, 6, 1000),    # GP19 (synthetic table) + NES, ragged count
    ((1, 1, 1, 0, 1), 1, 4, 1),       # one point, BRT06
])
def test_noalloc_matches_pooled_entry_twice(cuda, flags, brem, nq, n):
    import torch
    import bns_nurates_gb300 as bn
    from bns_nurates_gb300 import _capi as C
    lib = C.load()
    eos_h, m1_h = bn.synthetic_points(20261203, n, first=12345)
    eos, m1 = torch.from_numpy(eos_h).cuda(), torch.from_numpy(m1_h).cuda()
    f, p, q = bn.opacity_flags(*flags), bn.opacity_params(brem_implementation=brem), \
        bn.gauss_legendre(nq)
    stream = torch.cuda.current_stream().cuda_stream
    want = torch.empty((20, n), dtype=torch.float64, device="cuda")
    assert _call(lib.bnsn_m1_opacities, eos, m1, f, p, q, want, n, stream) == C.OK
    want_h = want.cpu().numpy()
    for _ in range(2):  # two calls in a row reuse the same static scratch
        got = torch.full((20, n), float("nan"), dtype=torch.float64, device="cuda")
        rc = _call(lib.bnsn_m1_opacities_noalloc, eos, m1, f, p, q, got, n, stream)
        assert rc == C.OK, lib.bnsn_last_error().decode()
        _assert_close(got.cpu().numpy(), want_h)


@pytest.mark.gpu
@pytest.mark.parametrize("brem,nq,n", [(2, 20, 4096), (0, 10, 777)])
def test_noalloc_mixed_after_other_inputs(cuda, brem, nq, n):
    """Mixed precision (its phase kernels pass flags and partial sums to each
    other through the scratch) with brem and NES on: a call on input set A
    leaves the static array full of A's records; the next call, on a
    different set B, must still equal the pooled entry on B."""
    import torch
    import bns_nurates_gb300 as bn
    from bns_nurates_gb300 import _capi as C
    lib = C.load()
    f, p, q = bn.opacity_flags(1, 1, 1, 1, 1), bn.opacity_params(brem_implementation=brem), \
        bn.gauss_legendre(nq)
    stream = torch.cuda.current_stream().cuda_stream
    sets = []
    for first in (0, 2 ** 22 + 17):   # A, then B (other points of the 256^3 workload)
        e_h, m_h = bn.synthetic_points(20261203, n, first=first)
        sets.append((torch.from_numpy(e_h).cuda(), torch.from_numpy(m_h).cuda()))
    (ea, ma), (eb, mb) = sets
    want = torch.empty((20, n), dtype=torch.float64, device="cuda")
    assert _call(lib.bnsn_m1_opacities, eb, mb, f, p, q, want, n, stream, C.MIXED) == C.OK
    junk = torch.empty((20, n), dtype=torch.float64, device="cuda")
    assert _call(lib.bnsn_m1_opacities_noalloc, ea, ma, f, p, q, junk, n, stream,
                 C.MIXED) == C.OK
    got = torch.full((20, n), float("nan"), dtype=torch.float64, device="cuda")
    rc = _call(lib.bnsn_m1_opacities_noalloc, eb, mb, f, p, q, got, n, stream, C.MIXED)
    assert rc == C.OK, lib.bnsn_last_error().decode()
    _assert_close(got.cpu().numpy(), want.cpu().numpy())


FRESH = textwrap.dedent("""
    import ctypes, sys
    import numpy as np
    import torch
    sys.path.insert(0, {repo!r})
    sys.path.insert(0, {tests!r})
    import bns_nurates_gb300 as bn
    from bns_nurates_gb300 import _capi as C
    from test_zz_no_alloc import _call
    lib = C.load()
    n = 2048
    e_h, m_h = bn.synthetic_points(31, n, first=999)
    e, m = torch.from_numpy(e_h).cuda(), torch.from_numpy(m_h).cuda()
    f, p, q = bn.opacity_flags(1, 1, 1, 1, 1), bn.opacity_params(), bn.gauss_legendre(10)
    s = torch.cuda.current_stream().cuda_stream
    outs = []
    for k in range(2):
        o = torch.full((20, n), float("nan"), dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        free0 = torch.cuda.mem_get_info()[0]
        rc = _call(lib.bnsn_m1_opacities_noalloc, e, m, f, p, q, o, n, s, C.MIXED)
        assert rc == C.OK, lib.bnsn_last_error().decode()
        torch.cuda.synchronize()
        free1 = torch.cuda.mem_get_info()[0]
        outs.append(o.cpu().numpy())
    np.savez({path!r}, first=outs[0], second=outs[1], free0=free0, free1=free1)
""")


@pytest.mark.gpu
def test_noalloc_as_first_call_of_a_fresh_process(cuda, tmp_path):
    """In a new process the no-alloc entry is the first opacity call (no
    per-device state, no pool yet).  Its two results equal the pooled entry's,
    and the second, warmed-up call leaves the device's free memory unchanged."""
    import torch
    import bns_nurates_gb300 as bn
    from bns_nurates_gb300 import _capi as C
    path = str(tmp_path / "fresh.npz")
    code = FRESH.format(repo=REPO, tests=os.path.join(REPO, "tests"), path=path)
    subprocess.run([sys.executable, "-c", code], check=True, timeout=600)
    r = np.load(path)
    n = 2048
    e_h, m_h = bn.synthetic_points(31, n, first=999)
    want = bn.m1_opacities(torch.from_numpy(e_h).cuda(), torch.from_numpy(m_h).cuda(),
                           bn.opacity_flags(1, 1, 1, 1, 1), bn.opacity_params(),
                           bn.gauss_legendre(10), precision="mixed").cpu().numpy()
    _assert_close(r["first"], want)
    _assert_close(r["second"], want)
    assert int(r["free1"]) == int(r["free0"]), (int(r["free0"]), int(r["free1"]))


@pytest.mark.gpu
def test_noalloc_empty_batch_sets_up_device(cuda):
    """npts = 0 is the set-up call a caller makes before stream capture."""
    import torch
    import bns_nurates_gb300 as bn
    from bns_nurates_gb300 import _capi as C
    eos = torch.zeros((11, 1), dtype=torch.float64, device="cuda")
    m1 = torch.zeros((12, 1), dtype=torch.float64, device="cuda")
    out = torch.zeros((20, 1), dtype=torch.float64, device="cuda")
    rc = _call(C.load().bnsn_m1_opacities_noalloc, eos, m1, bn.opacity_flags(),
               bn.opacity_params(), bn.gauss_legendre(4), out, 0, None)
    assert rc == C.OK
    assert torch.count_nonzero(out).item() == 0
