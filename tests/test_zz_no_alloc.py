"""bnsn_m1_opacities_noalloc: grey opacities with scratch in a static device
array, called through the C ABI and compared with bnsn_m1_opacities.

Collected last (file name) so it also runs after every other GPU test has
used the library in the same process; it passes on its own as well.
"""

import ctypes

import numpy as np
import pytest

TOL = 1e-12


def _call(entry, eos, m1, flags, params, q, out, n, stream):
    from bns_nurates_gb300 import api
    E, M, O = api._eos_soa(eos), api._m1_soa(m1), api._grey_soa(out)
    return entry(ctypes.byref(q), ctypes.byref(q), ctypes.byref(flags), ctypes.byref(params),
                 ctypes.byref(E), ctypes.byref(M), None, 1, 0, ctypes.byref(O), n, stream)


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
        g = got.cpu().numpy()
        assert np.all(np.isfinite(g) == np.isfinite(want_h))
        both = np.isfinite(g) & np.isfinite(want_h)
        d = np.abs(g - want_h)[both]
        scale = np.abs(want_h)[both]
        assert np.all(d <= TOL * scale), float(np.max(d / np.where(scale > 0, scale, 1)))


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
