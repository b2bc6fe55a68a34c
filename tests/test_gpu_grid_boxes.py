"""Grid boxes with ghost zones (bnsn_m1_opacities_grid_boxes) give, cell by
cell, the batched entry point's results on the same points; ghost cells are
left untouched; unit factors convert on the way in and out."""

import numpy as np
import pytest

import bns_nurates_gb300 as bn

pytestmark = pytest.mark.gpu

SHAPES = [((9, 7, 5), (2, 1, 1), (7, 6, 4)),     # (nx, ny, nz), lo, hi
          ((6, 5, 4), (1, 1, 1), (5, 4, 3)),
          ((3, 3, 3), (1, 1, 1), (1, 3, 3))]    # empty interior


def _boxes(torch, seed):
    boxes, packed_e, packed_m = [], [], []
    first = 0
    for (nx, ny, nz), lo, hi in SHAPES:
        n_in = (hi[0] - lo[0]) * (hi[1] - lo[1]) * (hi[2] - lo[2])
        e, m = bn.synthetic_points(seed, max(n_in, 1), first=first)
        first += n_in
        eos = np.full((11, nz, ny, nx), np.nan)
        m1 = np.full((12, nz, ny, nx), np.nan)
        if n_in:
            sl = (slice(None), slice(lo[2], hi[2]), slice(lo[1], hi[1]), slice(lo[0], hi[0]))
            shp = (hi[2] - lo[2], hi[1] - lo[1], hi[0] - lo[0])
            eos[sl] = e[:, :n_in].reshape((11,) + shp)
            m1[sl] = m[:, :n_in].reshape((12,) + shp)
            packed_e.append(e[:, :n_in])
            packed_m.append(m[:, :n_in])
        out = torch.full((20, nz, ny, nx), -7.0, dtype=torch.float64, device="cuda")
        boxes.append(dict(eos=torch.from_numpy(eos).cuda(), m1=torch.from_numpy(m1).cuda(),
                          out=out, lo=lo, hi=hi))
    return boxes, np.concatenate(packed_e, axis=1), np.concatenate(packed_m, axis=1)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_boxes_equal_batched_points(cuda, precision):
    torch = cuda
    boxes, pe, pm = _boxes(torch, 5)
    flags, params, q = bn.opacity_flags(), bn.opacity_params(), bn.gauss_legendre(6)
    bn.m1_opacities_grid_boxes(boxes, flags, params, q, precision=precision)
    want = bn.m1_opacities(torch.from_numpy(pe).cuda(), torch.from_numpy(pm).cuda(), flags,
                           params, q, precision=precision)
    torch.cuda.synchronize()
    want = want.cpu().numpy()
    k = 0
    for bx, ((nx, ny, nz), lo, hi) in zip(boxes, SHAPES):
        o = bx["out"].cpu().numpy()
        inner = np.zeros(o.shape[1:], dtype=bool)
        inner[lo[2]:hi[2], lo[1]:hi[1], lo[0]:hi[0]] = True
        n_in = int(inner.sum())
        got = o[:, inner]                       # (20, n_in) in z, y, x order
        np.testing.assert_array_equal(got, want[:, k:k + n_in])
        assert (o[:, ~inner] == -7.0).all(), "a ghost cell was written"
        k += n_in


def test_unit_factors(cuda):
    torch = cuda
    boxes, pe, pm = _boxes(torch, 9)
    # the host code holds nb in cm^-3 and wants kappa in cm^-1
    in_scale = [1e-21] + [1.] * 22
    out_scale = [1.] * 4 + [1e7] * 4 + [1.] * 4 + [1e7] * 8
    for bx in boxes:
        bx["eos"][0] *= 1e21
    flags, params, q = bn.opacity_flags(), bn.opacity_params(), bn.gauss_legendre(6)
    bn.m1_opacities_grid_boxes(boxes, flags, params, q, in_scale=in_scale, out_scale=out_scale)
    want = bn.m1_opacities(torch.from_numpy(pe).cuda(), torch.from_numpy(pm).cuda(), flags,
                           params, q).cpu().numpy() * np.array(out_scale)[:, None]
    (nx, ny, nz), lo, hi = SHAPES[0]
    o = boxes[0]["out"].cpu().numpy()[:, lo[2]:hi[2], lo[1]:hi[1], lo[0]:hi[0]]
    n0 = o[0].size
    # nb round-trips through two roundings (x 1e21, x 1e-21)
    np.testing.assert_allclose(o.reshape(20, -1), want[:, :n0], rtol=1e-10)
