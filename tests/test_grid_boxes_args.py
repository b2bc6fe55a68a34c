"""bnsn_m1_opacities_grid_boxes rejects bad box extents and missing fields
before touching a device (host-side checks), and an empty set of interiors
is a no-op."""

import ctypes

import bns_nurates_gb300 as bn
from bns_nurates_gb300 import _capi as C


def _call(boxes):
    arr = (C.GridBox * max(1, len(boxes)))(*boxes)
    q = bn.gauss_legendre(4)
    return C.load().bnsn_m1_opacities_grid_boxes(
        ctypes.byref(q), ctypes.byref(q), ctypes.byref(bn.opacity_flags()),
        ctypes.byref(bn.opacity_params()), arr, len(boxes), None, None, 1, 0, None)


def _box(shape=(4, 3, 2), lo=(1, 1, 0), hi=(3, 2, 2), fields=True):
    b = C.GridBox()
    b.shape[:], b.lo[:], b.hi[:] = list(shape), list(lo), list(hi)
    if fields:
        for f in range(11):
            b.eos[f] = 0x1000 + 8 * f
        for f in range(12):
            b.m1[f] = 0x2000 + 8 * f
        for f in range(20):
            b.out[f] = 0x3000 + 8 * f
    return b


def test_empty_interiors_are_a_no_op():
    assert _call([]) == 0
    assert _call([_box(lo=(2, 1, 0), hi=(2, 3, 2), fields=False)]) == 0


def test_bad_extents_rejected():
    assert _call([_box(lo=(3, 0, 0), hi=(2, 3, 2))]) == 1       # lo > hi
    assert _call([_box(hi=(5, 3, 2))]) == 1                      # hi > shape
    assert _call([_box(lo=(-1, 0, 0))]) == 1
    assert _call([_box(shape=(0, 3, 2), lo=(0, 0, 0), hi=(0, 3, 2))]) == 1


def test_missing_fields_rejected():
    b = _box()
    b.m1[5] = None
    assert _call([b]) == 1
    assert "m1 field" in C.load().bnsn_last_error().decode()
    b = _box()
    b.eos[8] = None          # mu_mu is optional; the device is not reached with bad precision
    arr = (C.GridBox * 1)(b)
    q = bn.gauss_legendre(4)
    rc = C.load().bnsn_m1_opacities_grid_boxes(
        ctypes.byref(q), ctypes.byref(q), ctypes.byref(bn.opacity_flags()),
        ctypes.byref(bn.opacity_params()), arr, 1, None, None, 1, 7, None)
    assert rc == 1 and "precision" in C.load().bnsn_last_error().decode()
