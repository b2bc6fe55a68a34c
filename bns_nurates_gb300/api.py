"""Python host API over the C ABI.

Batched calls take field-major structure-of-arrays tensors on the GPU:
``eos`` [11, N] in MyEOSParams field order (nb, temp, ye, yp, yn, mu_p, mu_n,
mu_e, mu_mu, dU, dm_eff), ``m1`` [12, N] = n[4], J[4], chi[4], optional
``distr`` [28, N] in NuDistributionParams order.  Grey results are [20, N] in
M1Opacities order (eta_0[4], kappa_0_a[4], eta[4], kappa_a[4], kappa_s[4]);
spectral results [16, N, n_energies] (j, kappa, j_s, kappa_s).

The per-point helpers ``ComputeM1Opacities`` / ``ComputeSpectralOpacities*``
keep the reference's names and arguments (m1_opacities.hpp:1297-1313,
1506-1660) and return the reference's result structs as dicts.

Nothing here computes physics: every number comes from the CUDA library, and
the module raises if that library is missing.
"""

import ctypes
import os

import numpy as np

from . import _capi as C


class BnsnError(RuntimeError):
    """A C-ABI call returned a non-zero bnsn_status."""

    def __init__(self, status):
        lib = C.load()
        msg = lib.bnsn_last_error().decode() or lib.bnsn_status_string(status).decode()
        super().__init__(f"bnsn status {status}: {msg}")
        self.status = status


def _check(status):
    if status != C.OK:
        raise BnsnError(status)


def _addr(t, k=None):
    """Device/host address of row k of a 2-D tensor/array (or of the array)."""
    if hasattr(t, "data_ptr"):
        base, stride = t.data_ptr(), (t.stride(0) * t.element_size() if t.dim() > 1 else 0)
    else:
        base = t.ctypes.data
        stride = t.strides[0] if t.ndim > 1 else 0
    return base if k is None else base + k * stride


def _stream_handle(stream):
    if stream is None:
        import torch
        return torch.cuda.current_stream().cuda_stream
    return getattr(stream, "cuda_stream", stream)


# ---------------------------------------------------------------------------
# struct helpers
# ---------------------------------------------------------------------------

def gauss_legendre(n):
    """MyQuadrature with n Gauss-Legendre nodes on [0, 1] (GaussLegendre)."""
    q = C.MyQuadrature()
    q.nx = n
    _check(C.load().bnsn_gauss_legendre(ctypes.byref(q)))
    return q


def opacity_flags(use_abs_em=1, use_pair=1, use_brem=1, use_inelastic_scatt=1, use_iso=1):
    return C.OpacityFlags(int(use_abs_em), int(use_pair), int(use_brem),
                          int(use_inelastic_scatt), int(use_iso))


def opacity_params(use_dU=True, use_dm_eff=False, use_WM_ab=True, use_WM_sc=True,
                   use_decay=True, brem_implementation=C.BREM_HR98, use_NN_medium_corr=True,
                   neglect_blocking=False):
    return C.OpacityParams(bool(use_dU), bool(use_dm_eff), bool(use_WM_ab), bool(use_WM_sc),
                           bool(use_decay), int(brem_implementation),
                           bool(use_NN_medium_corr), bool(neglect_blocking))


def flags_tuple(f):
    return (f.use_abs_em, f.use_pair, f.use_brem, f.use_inelastic_scatt, f.use_iso)


def params_tuple(p):
    return (int(p.use_dU), int(p.use_dm_eff), int(p.use_WM_ab), int(p.use_WM_sc),
            int(p.use_decay), int(p.brem_implementation), int(p.use_NN_medium_corr),
            int(p.neglect_blocking))


def quad_arrays(q):
    n = q.nx
    return np.array(q.points[:n]), np.array(q.w[:n])


def _eos_soa(eos):
    return C.EosSoA(*[_addr(eos, k) for k in range(11)])


def _m1_soa(m1):
    s = C.M1SoA()
    for k in range(4):
        s.n[k], s.J[k], s.chi[k] = _addr(m1, k), _addr(m1, 4 + k), _addr(m1, 8 + k)
    return s


def _distr_soa(d):
    s = C.DistrSoA()
    for q, name in enumerate(("w_t", "temp_t", "eta_t", "w_f", "temp_f", "c_f", "beta_f")):
        arr = getattr(s, name)
        for k in range(4):
            arr[k] = _addr(d, 4 * q + k)
    return s


def _grey_soa(out):
    s = C.M1OpacitiesSoA()
    for q, name in enumerate(("eta_0", "kappa_0_a", "eta", "kappa_a", "kappa_s")):
        arr = getattr(s, name)
        for k in range(4):
            arr[k] = _addr(out, 4 * q + k)
    return s


def _spec_soa(out):
    s = C.SpectralSoA()
    for q, name in enumerate(("j", "kappa", "j_s", "kappa_s")):
        arr = getattr(s, name)
        for k in range(4):
            arr[k] = _addr(out, 4 * q + k)
    return s


def _prec(precision):
    return {"fp64": C.FP64, "mixed": C.MIXED, C.FP64: C.FP64, C.MIXED: C.MIXED}[precision]


# ---------------------------------------------------------------------------
# batched device API
# ---------------------------------------------------------------------------

def m1_opacities(eos, m1, flags, params, quad_1d, quad_2d=None, distr=None, stim_abs=1,
                 precision="fp64", out=None, stream=None):
    """Grey M1 opacities of N points (tensors on the current CUDA device)."""
    import torch
    n = eos.shape[1]
    assert eos.shape[0] == 11 and m1.shape == (12, n)
    assert eos.is_cuda and m1.is_cuda and eos.dtype == torch.float64
    assert eos.stride(1) == 1 and m1.stride(1) == 1
    if out is None:
        out = torch.empty((20, n), dtype=torch.float64, device=eos.device)
    quad_2d = quad_1d if quad_2d is None else quad_2d
    E, M, O = _eos_soa(eos), _m1_soa(m1), _grey_soa(out)
    D = None if distr is None else _distr_soa(distr)
    _check(C.load().bnsn_m1_opacities(
        ctypes.byref(quad_1d), ctypes.byref(quad_2d), ctypes.byref(flags), ctypes.byref(params),
        ctypes.byref(E), ctypes.byref(M), None if D is None else ctypes.byref(D),
        int(stim_abs), _prec(precision), ctypes.byref(O), n, _stream_handle(stream)))
    return out


def m1_opacities_grid_boxes(boxes, flags, params, quad_1d, quad_2d=None, in_scale=None,
                            out_scale=None, stim_abs=1, precision="fp64", stream=None):
    """Grey opacities of the interiors of grid boxes (bnsn_m1_opacities_grid_boxes).

    boxes: dicts with "eos" [11, nz, ny, nx], "m1" [12, nz, ny, nx] and "out"
    [20, nz, ny, nx] contiguous float64 CUDA tensors (a field per leading
    index) and the interior "lo", "hi" as (i, j, k) index triples (x first).
    in_scale (23) / out_scale (20): optional unit factors."""
    arr = (C.GridBox * max(1, len(boxes)))()
    for b, bx in enumerate(boxes):
        eos, m1, out = bx["eos"], bx["m1"], bx["out"]
        nz, ny, nx = eos.shape[1:]
        for t, n_f in ((eos, 11), (m1, 12), (out, 20)):
            if tuple(t.shape) != (n_f, nz, ny, nx) or not t.is_contiguous():
                raise ValueError("box fields must be contiguous [fields, nz, ny, nx] tensors")
        arr[b].shape[:] = [nx, ny, nz]
        arr[b].lo[:] = [int(v) for v in bx["lo"]]
        arr[b].hi[:] = [int(v) for v in bx["hi"]]
        for f in range(11):
            arr[b].eos[f] = _addr(eos, f)
        for f in range(12):
            arr[b].m1[f] = _addr(m1, f)
        for f in range(20):
            arr[b].out[f] = _addr(out, f)
    q2 = quad_1d if quad_2d is None else quad_2d
    sin = None if in_scale is None else (ctypes.c_double * 23)(*[float(v) for v in in_scale])
    sout = None if out_scale is None else (ctypes.c_double * 20)(*[float(v) for v in out_scale])
    _check(C.load().bnsn_m1_opacities_grid_boxes(
        ctypes.byref(quad_1d), ctypes.byref(q2), ctypes.byref(flags), ctypes.byref(params), arr,
        len(boxes), sin, sout, int(stim_abs), _prec(precision), _stream_handle(stream)))


def spectral_opacities(eos, m1, flags, params, quad_1d, energies, distr=None, stimulated=1,
                       precision="fp64", out=None, stream=None):
    """Spectral opacities of N points at the given energies: [16, N, n_e]."""
    import torch
    n = eos.shape[1]
    e = np.ascontiguousarray(np.asarray(energies, dtype=np.float64))
    if out is None:
        out = torch.empty((16, n, e.size), dtype=torch.float64, device=eos.device)
    E, M, O = _eos_soa(eos), _m1_soa(m1), _spec_soa(out)
    D = None if distr is None else _distr_soa(distr)
    _check(C.load().bnsn_spectral_opacities(
        ctypes.byref(quad_1d), ctypes.byref(flags), ctypes.byref(params), ctypes.byref(E),
        ctypes.byref(M), None if D is None else ctypes.byref(D), e.ctypes.data, e.size,
        int(stimulated), _prec(precision), ctypes.byref(O), n, _stream_handle(stream)))
    return out


def distr_from_m1(m1, out=None, stream=None):
    """CalculateDistrParamsFromM1 for N points: [28, N]."""
    import torch
    n = m1.shape[1]
    if out is None:
        out = torch.empty((28, n), dtype=torch.float64, device=m1.device)
    _check(C.load().bnsn_distr_from_m1(ctypes.byref(_m1_soa(m1)), ctypes.byref(_distr_soa(out)),
                                       n, _stream_handle(stream)))
    return out


def nu_equilibrium(eos, stream=None):
    """NuEquilibriumParams + ComputeM1DensitiesEq: (distr [28, N], m1 [12, N])."""
    import torch
    n = eos.shape[1]
    distr = torch.empty((28, n), dtype=torch.float64, device=eos.device)
    m1 = torch.empty((12, n), dtype=torch.float64, device=eos.device)
    arr = ctypes.c_void_p * 4
    nn = arr(*[_addr(m1, k) for k in range(4)])
    jj = arr(*[_addr(m1, 4 + k) for k in range(4)])
    cc = arr(*[_addr(m1, 8 + k) for k in range(4)])
    _check(C.load().bnsn_nu_equilibrium(ctypes.byref(_eos_soa(eos)),
                                        ctypes.byref(_distr_soa(distr)), nn, jj, cc, n,
                                        _stream_handle(stream)))
    return distr, m1


# Reference names of the Fermi-Dirac integral family (functions.hpp:442-4375)
# by twice the order.
FDI_NAMES = {-9: "FDI_m92", -7: "FDI_m72", -5: "FDI_m52", -3: "FDI_m32", -1: "FDI_m12",
             0: "FDI_0", 1: "FDI_p12", 2: "FDI_p1", 3: "FDI_p32", 4: "FDI_p2", 5: "FDI_p52",
             6: "FDI_p3", 7: "FDI_p72", 8: "FDI_p4", 9: "FDI_p92", 10: "FDI_p5",
             11: "FDI_p112", 12: "FDI_p6", 13: "FDI_p132", 14: "FDI_p7", 15: "FDI_p152",
             16: "FDI_p8", 17: "FDI_p172", 18: "FDI_p9", 19: "FDI_p192", 20: "FDI_p10",
             21: "FDI_p212"}


def _twice_order(order):
    k2 = int(round(2 * float(order)))
    if k2 != 2 * float(order) or k2 not in FDI_NAMES:
        raise ValueError("order must be one of -9/2, -7/2, ..., -1/2, 0, 1/2, 1, ..., 21/2")
    return k2


def fdi(order, x, out=None, stream=None):
    """Fermi-Dirac integral F_order(x) of a float64 CUDA tensor, unnormalised as
    the reference's FDI_* functions (order = -9/2 .. -1/2 or 0 .. 21/2 in
    halves)."""
    import torch
    k2 = _twice_order(order)
    if x.dtype != torch.float64 or not x.is_cuda:
        raise ValueError("x must be a float64 CUDA tensor")
    x = x.contiguous()
    if out is None:
        out = torch.empty_like(x)
    _check(C.load().bnsn_fdi(k2, x.data_ptr(), out.data_ptr(), x.numel(),
                             _stream_handle(stream)))
    return out


def pair_j_mixed(y, z, eta, stream=None):
    """The mixed path's pair integrals J_0 = PairPsi(y, z) / (1 - e^{y+z}) and
    J_1 = PairPsi(z, y) / (1 - e^{y+z}) at float64 CUDA tensors y, z, eta of one
    shape: (j0, j1, lscale) with J_l = exp(lscale) * j_l."""
    import torch
    y, z, eta = (torch.broadcast_tensors(*(t.to(torch.float64) for t in (y, z, eta))))
    y, z, eta = y.contiguous(), z.contiguous(), eta.contiguous()
    if not y.is_cuda:
        raise ValueError("y, z, eta must be CUDA tensors")
    j0, j1, ls = torch.empty_like(y), torch.empty_like(y), torch.empty_like(y)
    _check(C.load().bnsn_pair_j_mixed(y.data_ptr(), z.data_ptr(), eta.data_ptr(), j0.data_ptr(),
                                      j1.data_ptr(), ls.data_ptr(), y.numel(),
                                      _stream_handle(stream)))
    return j0, j1, ls


def nes_m_mixed(w, wp, eta, stream=None):
    """The mixed path's NES/NPS out-kernel integrals: MezzacappaIntOut(w, w',
    b1, b2) = exp(lscale) * (b1 m1 + b2 m2) at float64 CUDA tensors w, w', eta
    of one shape: (m1, m2, lscale)."""
    import torch
    w, wp, eta = (torch.broadcast_tensors(*(t.to(torch.float64) for t in (w, wp, eta))))
    w, wp, eta = w.contiguous(), wp.contiguous(), eta.contiguous()
    if not w.is_cuda:
        raise ValueError("w, wp, eta must be CUDA tensors")
    m1, m2, ls = torch.empty_like(w), torch.empty_like(w), torch.empty_like(w)
    _check(C.load().bnsn_nes_m_mixed(w.data_ptr(), wp.data_ptr(), eta.data_ptr(), m1.data_ptr(),
                                     m2.data_ptr(), ls.data_ptr(), w.numel(),
                                     _stream_handle(stream)))
    return m1, m2, ls


def fdi_host(order, x):
    """F_order(x) of a host float64 array (copied to the GPU and back)."""
    k2 = _twice_order(order)
    x = np.ascontiguousarray(x, dtype=np.float64)
    out = np.empty_like(x)
    _check(C.load().bnsn_fdi_host(k2, x.ctypes.data, out.ctypes.data, x.size))
    return out


def set_gp19_table(tab):
    """Load a GP19 table dict (dims, nb, ye, t, w, [lognb, logw], data)."""
    dims = (ctypes.c_int * 4)(*tab["dims"])
    arrs = [np.ascontiguousarray(tab[k], dtype=np.float64) if tab.get(k) is not None else None
            for k in ("nb", "ye", "t", "w", "lognb", "logw", "data")]
    ptrs = [None if a is None else a.ctypes.data for a in arrs]
    _check(C.load().bnsn_gp19_set_table(dims, *ptrs))


def load_gp19_header(path):
    """Load a GP19 table from a header in the reference's GP19Table.hpp format."""
    _check(C.load().bnsn_gp19_load_header(os.fsencode(path)))


_GP19_DIMS = ("GP19_nb_dims", "GP19_Ye_dims", "GP19_T_dims", "GP19_w_dims")
_GP19_ARRAYS = (("nb", "GP19_nb_axis"), ("ye", "GP19_Ye_axis"), ("t", "GP19_T_axis"),
                ("w", "GP19_w_axis"), ("lognb", "GP19_lognb_axis"),
                ("logw", "GP19_logw_axis"), ("data", "GP19_data"))


def gp19_table_from_header(path):
    """Parse a header in the reference's GP19Table.hpp format into the table
    dict of set_table (host only; the same declarations bnsn_gp19_load_header
    reads)."""
    import re
    text = open(path).read()
    text = re.sub(r"/\*.*?\*/", " ", text, flags=re.S)
    text = re.sub(r"//[^\n]*", " ", text)

    def decl(name):
        m = re.search(r"(?<![A-Za-z0-9_])" + name + r"(?![A-Za-z0-9_])\s*(\[[^\]]*\])?\s*=(?!=)",
                      text)
        return None if m is None else m.end()

    dims = []
    for name in _GP19_DIMS:
        q = decl(name)
        if q is None:
            raise ValueError(f"{name} not declared in {path}")
        dims.append(int(re.match(r"\s*(\d+)", text[q:]).group(1)))
    tab = {"dims": tuple(dims)}
    num = r"[-+]?(?:\d+\.?\d*|\.\d+)(?:[eE][-+]?\d+)?"
    for key, name in _GP19_ARRAYS:
        q = decl(name)
        if q is None:
            tab[key] = None
            continue
        depth, i = 0, text.index("{", q)
        for j in range(i, len(text)):
            depth += {"{": 1, "}": -1}.get(text[j], 0)
            if depth == 0:
                break
        tab[key] = np.array([float(v) for v in re.findall(num, text[i:j + 1])])
    for key, n in (("nb", dims[0]), ("ye", dims[1]), ("t", dims[2]), ("w", dims[3]),
                   ("data", dims[0] * dims[1] * dims[2] * dims[3])):
        if tab[key] is None or tab[key].size != n:
            raise ValueError(f"GP19 {key} array missing or of the wrong length in {path}")
    return tab


def synthetic_points(seed, n, first=0, nthreads=0):
    """Seeded synthetic points on the host: (eos [11, n], m1 [12, n]) numpy."""
    import os
    eos = np.empty((11, n))
    m1 = np.empty((12, n))
    _check(C.load().bnsn_synthetic_points(seed, first, n, eos.ctypes.data, m1.ctypes.data,
                                          int(nthreads or os.cpu_count())))
    return eos, m1


def fp64_peak_tflops(iters=1 << 16):
    """Measured FP64 FMA throughput of the current device (TFLOP/s)."""
    v = ctypes.c_double()
    _check(C.load().bnsn_fp64_peak_probe(int(iters), ctypes.byref(v)))
    return v.value


def fp32_peak_tflops(iters=1 << 18):
    """Measured FP32 FMA throughput of the current device (TFLOP/s)."""
    v = ctypes.c_double()
    _check(C.load().bnsn_fp32_peak_probe(int(iters), ctypes.byref(v)))
    return v.value


def phase_timing(enable):
    """Bracket every library kernel launch with CUDA events (diagnostic)."""
    _check(C.load().bnsn_phase_timing(int(bool(enable))))


def phase_times():
    """Per-phase device ms and launch counts since the previous call."""
    ms = (ctypes.c_double * C.NUM_PHASES)()
    n = (ctypes.c_int64 * C.NUM_PHASES)()
    _check(C.load().bnsn_phase_times(ms, n))
    return {name: (ms[k], n[k]) for k, name in enumerate(C.PHASES)}


def kernel_launches():
    """Kernels launched by the library in this process."""
    return int(C.load().bnsn_kernel_launches())


def spectral_mixed_stats(reset=False):
    """Mixed spectral path on the current device since the last reset:
    {"evaluated", "fp64", "pb_fp64", "nes_fp64"} (point, energy) counts."""
    c = (ctypes.c_int64 * 4)()
    _check(C.load().bnsn_spectral_mixed_stats(c, int(reset)))
    return dict(zip(("evaluated", "fp64", "pb_fp64", "nes_fp64"), (int(v) for v in c)))


def grey_mixed_stats(reset=False):
    """Mixed grey path on the current device since the last reset:
    {"evaluated", "nes_df", "nes_fp64", "pair_fp64", "brem_fp64"} point counts."""
    c = (ctypes.c_int64 * 5)()
    _check(C.load().bnsn_grey_mixed_stats(c, int(reset)))
    return dict(zip(("evaluated", "nes_df", "nes_fp64", "pair_fp64", "brem_fp64"),
                    (int(v) for v in c)))


def nonfinite_outputs(reset=False):
    """Outputs with a NaN or Inf on the current device since the last reset:
    {"grey_points", "spectral_pairs"}."""
    c = (ctypes.c_int64 * 2)()
    _check(C.load().bnsn_nonfinite_outputs(c, int(reset)))
    return {"grey_points": int(c[0]), "spectral_pairs": int(c[1])}


def m1_opacities_host(eos, m1, flags, params, quad_1d, quad_2d=None, stim_abs=1,
                      precision="fp64", out=None):
    """Grey opacities of host (numpy or pinned torch) arrays, copies included."""
    n = eos.shape[1]
    if out is None:
        out = np.empty((20, n))
    quad_2d = quad_1d if quad_2d is None else quad_2d
    _check(C.load().bnsn_m1_opacities_host(
        ctypes.byref(quad_1d), ctypes.byref(quad_2d), ctypes.byref(flags), ctypes.byref(params),
        ctypes.byref(_eos_soa(eos)), ctypes.byref(_m1_soa(m1)), int(stim_abs),
        _prec(precision), ctypes.byref(_grey_soa(out)), n))
    return out


# ---------------------------------------------------------------------------
# per-point mirrors of the reference functions
# ---------------------------------------------------------------------------

def _struct_dict(s):
    return {name: list(getattr(s, name)) for name, _ in s._fields_}


def ComputeM1Opacities(quad_1d, quad_2d, grey_pars):
    """ComputeM1Opacities(quad_1d, quad_2d, grey_pars) -> M1Opacities dict."""
    o = C.M1Opacities()
    _check(C.load().bnsn_compute_m1_opacities_point(
        ctypes.byref(quad_1d), ctypes.byref(quad_2d), ctypes.byref(grey_pars), 1, ctypes.byref(o)))
    return _struct_dict(o)


def ComputeM1OpacitiesNotStimulated(quad_1d, quad_2d, grey_pars):
    o = C.M1Opacities()
    _check(C.load().bnsn_compute_m1_opacities_point(
        ctypes.byref(quad_1d), ctypes.byref(quad_2d), ctypes.byref(grey_pars), 0, ctypes.byref(o)))
    return _struct_dict(o)


def ComputeSpectralOpacitiesStimulatedAbs(nu, quad_1d, grey_pars):
    o = C.SpectralOpacities()
    _check(C.load().bnsn_compute_spectral_opacities_point(
        float(nu), ctypes.byref(quad_1d), ctypes.byref(grey_pars), 1, ctypes.byref(o)))
    return _struct_dict(o)


def ComputeSpectralOpacitiesNotStimulatedAbs(nu, quad_1d, grey_pars):
    o = C.SpectralOpacities()
    _check(C.load().bnsn_compute_spectral_opacities_point(
        float(nu), ctypes.byref(quad_1d), ctypes.byref(grey_pars), 0, ctypes.byref(o)))
    return _struct_dict(o)


# ---------------------------------------------------------------------------
# batched AMR blocks
# ---------------------------------------------------------------------------

class BlocksPlan:
    """Planned grey opacities of many AMR blocks (bnsn_blocks_plan_create /
    bnsn_blocks_run).  `blocks` is a sequence of (first, count, flags, brem,
    nquad) with flags a 5-tuple (abs_em, pair, brem, inelastic, iso); eos [11,
    N], m1 [12, N] and out [20, N] are CUDA tensors holding every block's
    points."""

    def __init__(self, blocks, eos, m1, out, params=None, stim_abs=1, precision="fp64",
                 tune=False, stream=None):
        lib = C.load()
        arr = (C.Block * max(1, len(blocks)))()
        for k, (first, count, flags, brem, nq) in enumerate(blocks):
            arr[k] = C.Block(int(first), int(count), opacity_flags(*flags), int(brem), int(nq))
        self._handle = ctypes.c_void_p()
        params = opacity_params() if params is None else params
        _check(lib.bnsn_blocks_plan_create(
            arr, len(blocks), ctypes.byref(params), int(stim_abs), _prec(precision), int(bool(tune)),
            ctypes.byref(_eos_soa(eos)), ctypes.byref(_m1_soa(m1)), ctypes.byref(_grey_soa(out)),
            _stream_handle(stream), ctypes.byref(self._handle)))

    def run(self, eos, m1, out, stream=None):
        _check(C.load().bnsn_blocks_run(self._handle, ctypes.byref(_eos_soa(eos)),
                                        ctypes.byref(_m1_soa(m1)), ctypes.byref(_grey_soa(out)),
                                        _stream_handle(stream)))
        return out

    def groups(self):
        lib = C.load()
        res = []
        for g in range(lib.bnsn_blocks_plan_groups(self._handle)):
            nq, rx, br = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
            n, ch, gs = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_double()
            _check(lib.bnsn_blocks_plan_info(self._handle, g, ctypes.byref(nq), ctypes.byref(rx),
                                             ctypes.byref(br), ctypes.byref(n), ctypes.byref(ch),
                                             ctypes.byref(gs)))
            res.append(dict(nquad=nq.value, reactions=rx.value, brem=br.value, npts=n.value,
                            chunk=ch.value, grid_scale=gs.value))
        return res

    def layout(self):
        """Steps per run, points per step and scratch bytes of the plan."""
        st, sp, nb = ctypes.c_int(), ctypes.c_int64(), ctypes.c_int64()
        _check(C.load().bnsn_blocks_plan_layout(self._handle, ctypes.byref(st), ctypes.byref(sp),
                                                ctypes.byref(nb)))
        return dict(steps=st.value, step_points=sp.value, scratch_bytes=nb.value)

    @staticmethod
    def set_options(scratch_bytes=0, step_points=0):
        """Options of plans created afterwards: the scratch limit in bytes (0:
        a quarter of the free device memory) and the points per step over all
        groups (0: the tuner's choice, or the default without tuning)."""
        _check(C.load().bnsn_blocks_set_options(int(scratch_bytes), int(step_points)))

    def close(self):
        if self._handle:
            C.load().bnsn_blocks_plan_destroy(self._handle)
            self._handle = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
