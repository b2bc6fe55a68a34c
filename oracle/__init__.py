"""CPU oracle for the bns_nurates opacity path (test infrastructure only).

Two implementations share one calling convention:

* ``port``: ``bnsn_oracle.c``, a plain-C restatement of the reference
  algorithm.  It builds anywhere (``build()``), including the GPU host.
* ``ref``: ``oracle/_ref/libbnsn_ref.so``, the reference headers themselves
  compiled by ``build_ref.py``.  It exists only where the reference checkout is
  present; tests use it to pin the port bit for bit.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg
use this package, as the checker; the product never imports it.
"""

import ctypes
import os
import platform
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_SO = os.path.join(HERE, "libbnsn_oracle.so")
# Same source with FMA contraction enabled: identical algorithm, different
# rounding.  Where the two builds disagree, the reference result itself is
# not reproducible to the last bits (cancellation), which the GPU parity
# tests use as the per-element conditioning of each output.
PORT_FMA_SO = os.path.join(HERE, "libbnsn_oracle_fma.so")
# Same source with every Fermi integral moved by one part in 2^52 (a bit of
# its argument picks the sign): the reference's sensitivity to an equally
# accurate evaluation of its Fermi integrals, which the catastrophic
# cancellation of the pair Psi polynomial at small y, z amplifies.
PORT_FDI_SO = os.path.join(HERE, "libbnsn_oracle_fdi.so")
REF_SO = os.path.join(HERE, "_ref", "libbnsn_ref.so")
REF_LAYOUT = os.path.join(HERE, "_ref", "ref_layout")

N_EOS, N_M1, N_DISTR, N_GREY, N_SPEC = 11, 12, 28, 20, 16


def build(force=False):
    """Compile the C oracle (always) and the reference build (when present)."""
    srcs = [os.path.join(HERE, "bnsn_oracle.c"), os.path.join(HERE, "bnsn_synth.c")]
    hdr = os.path.join(HERE, "bnsn_oracle_consts.h")
    stale = (not os.path.exists(PORT_SO)) or force or max(
        os.path.getmtime(f) for f in srcs + [hdr]) > os.path.getmtime(PORT_SO)
    if stale:
        subprocess.check_call([
            "gcc", "-std=c11", "-O2", "-ffp-contract=off", "-fopenmp", "-fPIC",
            "-shared"] + srcs + ["-o", PORT_SO, "-lm"])
    if stale or not os.path.exists(PORT_FMA_SO):
        fma = ["-mfma"] if platform.machine() in ("x86_64", "AMD64") else []
        subprocess.check_call([
            "gcc", "-std=c11", "-O2", "-ffp-contract=fast", "-fopenmp", "-fPIC",
            "-shared"] + fma + srcs + ["-o", PORT_FMA_SO, "-lm"])
    if stale or not os.path.exists(PORT_FDI_SO):
        subprocess.check_call([
            "gcc", "-std=c11", "-O2", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared",
            "-DORACLE_FDI_JITTER"] + srcs + ["-o", PORT_FDI_SO, "-lm"])
    from . import build_ref  # noqa: WPS433 (local import: optional step)
    try:
        build_ref.build()
    except Exception as exc:  # the reference is optional on a GPU host
        print(f"oracle: reference build skipped ({exc})")


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def _i32(vals):
    return np.ascontiguousarray(np.asarray(vals, dtype=np.int32))


def _f64(a):
    return np.ascontiguousarray(np.asarray(a, dtype=np.float64))


class Oracle:
    """ctypes view of one implementation (``prefix`` is ``oracle_`` or ``ref_``)."""

    def __init__(self, path, prefix):
        self.path = path
        self.prefix = prefix
        self.lib = ctypes.CDLL(path)
        self.kind = "port" if prefix == "oracle_" else "reference"

    def _f(self, name):
        return getattr(self.lib, self.prefix + name)

    # -- batch entry points ------------------------------------------------
    def gauss_legendre(self, n):
        x = np.zeros(n)
        w = np.zeros(n)
        f = self._f("gauss_legendre")
        f.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
        f(n, _p(x), _p(w))
        return x, w

    def m1_opacities(self, eos, m1, flags, pars, quad1, quad2=None, distr=None,
                     stim_abs=1, nthreads=None):
        eos, m1 = _f64(eos), _f64(m1)
        npts = eos.shape[1]
        assert eos.shape == (N_EOS, npts) and m1.shape == (N_M1, npts)
        quad2 = quad1 if quad2 is None else quad2
        x1, w1 = (_f64(v) for v in quad1)
        x2, w2 = (_f64(v) for v in quad2)
        d = None if distr is None else _f64(distr)
        out = np.zeros((N_GREY, npts))
        fl, pa = _i32(flags), _i32(pars)
        f = self._f("m1_opacities_batch")
        f.argtypes = [ctypes.c_int64] + [ctypes.c_void_p] * 5 + [
            ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
            ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
            ctypes.c_int, ctypes.c_void_p, ctypes.c_int]
        f.restype = ctypes.c_int
        rc = f(npts, _p(eos), _p(m1), None if d is None else _p(d), _p(fl), _p(pa),
               len(x1), _p(x1), _p(w1), len(x2), _p(x2), _p(w2), int(stim_abs),
               _p(out), int(nthreads or os.cpu_count()))
        if rc:
            raise RuntimeError(f"{self.prefix}m1_opacities_batch failed ({rc})")
        return out

    def spectral(self, eos, m1, flags, pars, quad, energies, distr=None,
                 stimulated=1, nthreads=None):
        eos, m1 = _f64(eos), _f64(m1)
        npts = eos.shape[1]
        x, w = (_f64(v) for v in quad)
        e = _f64(energies)
        d = None if distr is None else _f64(distr)
        out = np.zeros((N_SPEC, npts * len(e)))
        fl, pa = _i32(flags), _i32(pars)
        f = self._f("spectral_batch")
        f.argtypes = [ctypes.c_int64] + [ctypes.c_void_p] * 5 + [
            ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
            ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_int]
        f.restype = ctypes.c_int
        rc = f(npts, _p(eos), _p(m1), None if d is None else _p(d), _p(fl), _p(pa),
               len(x), _p(x), _p(w), len(e), _p(e), int(stimulated), _p(out),
               int(nthreads or os.cpu_count()))
        if rc:
            raise RuntimeError(f"{self.prefix}spectral_batch failed ({rc})")
        return out.reshape(N_SPEC, npts, len(e))

    def distr_from_m1(self, eos, m1):
        eos, m1 = _f64(eos), _f64(m1)
        npts = eos.shape[1]
        out = np.zeros((N_DISTR, npts))
        f = self._f("distr_from_m1_batch")
        f.argtypes = [ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
        f(npts, _p(eos), _p(m1), _p(out))
        return out

    def nu_equilibrium(self, eos):
        eos = _f64(eos)
        npts = eos.shape[1]
        distr = np.zeros((N_DISTR, npts))
        m1 = np.zeros((N_M1, npts))
        f = self._f("nu_equilibrium_batch")
        f.argtypes = [ctypes.c_int64] + [ctypes.c_void_p] * 3
        f(npts, _p(eos), _p(distr), _p(m1))
        return distr, m1

    def synthetic_points(self, seed, n, first=0, nthreads=None):
        """Port only: the seeded synthetic workload (eos [11, n], m1 [12, n]),
        bit-identical to the library's bnsn_synthetic_points."""
        eos = np.zeros((N_EOS, n))
        m1 = np.zeros((N_M1, n))
        f = self._f("synthetic_points")
        f.argtypes = [ctypes.c_uint64, ctypes.c_int64, ctypes.c_int64, ctypes.c_void_p,
                      ctypes.c_void_p, ctypes.c_int]
        f.restype = ctypes.c_int
        if f(int(seed), int(first), int(n), _p(eos), _p(m1), int(nthreads or os.cpu_count())):
            raise ValueError("synthetic_points: bad arguments")
        return eos, m1

    # -- unit-level entry points -------------------------------------------
    def fdi(self, k, x):
        x = _f64(x)
        out = np.zeros_like(x)
        f = self._f("fdi")
        f.argtypes = [ctypes.c_int, ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p]
        f(int(k), x.size, _p(x), _p(out))
        return out

    def pair_kernel(self, temp, mu_e, omega, omega_prime):
        out = np.zeros(8)
        f = self._f("pair_kernel")
        f.argtypes = [ctypes.c_double] * 4 + [ctypes.c_void_p]
        f(temp, mu_e, omega, omega_prime, _p(out))
        return out

    def brem_kernel(self, impl, eos11, omega, omega_prime, medium_corr=1):
        eos11 = _f64(eos11)
        out = np.zeros(2)
        f = self._f("brem_kernel")
        f.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_double,
                      ctypes.c_double, ctypes.c_int, ctypes.c_void_p]
        f(int(impl), _p(eos11), omega, omega_prime, int(medium_corr), _p(out))
        return out

    def inelastic_kernel(self, temp, mu_e, omega, omega_prime):
        out = np.zeros(8)
        f = self._f("inelastic_kernel")
        f.argtypes = [ctypes.c_double] * 4 + [ctypes.c_void_p]
        f(temp, mu_e, omega, omega_prime, _p(out))
        return out

    def abs_opacity(self, eos11, pars, omega, stimulated=0):
        eos11, pa = _f64(eos11), _i32(pars)
        out = np.zeros(4)
        f = self._f("abs_opacity")
        f.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_double,
                      ctypes.c_int, ctypes.c_void_p]
        f(_p(eos11), _p(pa), omega, int(stimulated), _p(out))
        return out

    def iso_scatt(self, eos11, pars, omega, l=0):
        eos11, pa = _f64(eos11), _i32(pars)
        out = np.zeros(2)
        f = self._f("iso_scatt")
        f.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_double,
                      ctypes.c_int, ctypes.c_void_p]
        f(_p(eos11), _p(pa), omega, int(l), _p(out))
        return out

    def weak_magnetism(self, omega):
        out = np.zeros(6)
        f = self._f("weak_magnetism")
        f.argtypes = [ctypes.c_double, ctypes.c_void_p]
        f(omega, _p(out))
        return out

    def total_nu_f(self, distr28, omega):
        d, om = _f64(distr28), _f64(omega)
        out = np.zeros((4, om.size))
        f = self._f("total_nu_f")
        f.argtypes = [ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p]
        f(_p(d), om.size, _p(om), _p(out))
        return out

    def special(self, which, a, b=None, c=None):
        a = _f64(a)
        b = _f64(a if b is None else b)
        c = _f64(a if c is None else c)
        out = np.zeros_like(a)
        f = self._f("special")
        f.argtypes = [ctypes.c_int, ctypes.c_int64] + [ctypes.c_void_p] * 4
        f(int(which), a.size, _p(a), _p(b), _p(c), _p(out))
        return out

    def set_gp19_table(self, tab):
        """Port only: load a GP19 table (the reference has it compiled in)."""
        assert self.prefix == "oracle_"
        dims = _i32(tab["dims"])
        arrs = [_f64(tab[k]) for k in ("nb", "ye", "t", "w", "lognb", "logw", "data")]
        f = self._f("gp19_set_table")
        f.argtypes = [ctypes.c_void_p] * 8
        f.restype = ctypes.c_int
        if f(_p(dims), *[_p(a) for a in arrs]):
            raise MemoryError("gp19 table")
        self._gp19_keep = arrs


_cache = {}


def port():
    """The C restatement (built on demand), with the synthetic GP19 table loaded."""
    if "port" not in _cache:
        if not os.path.exists(PORT_SO):
            build()
        o = Oracle(PORT_SO, "oracle_")
        o.set_gp19_table(_synthetic_gp19())
        _cache["port"] = o
    return _cache["port"]


def port_fma():
    """The C restatement compiled with FMA contraction (conditioning probe)."""
    if "port_fma" not in _cache:
        if not os.path.exists(PORT_FMA_SO):
            build()
        o = Oracle(PORT_FMA_SO, "oracle_")
        o.set_gp19_table(_synthetic_gp19())
        _cache["port_fma"] = o
    return _cache["port_fma"]


def port_fdi():
    """The C restatement with its Fermi integrals moved by one part in 2^52
    (conditioning probe)."""
    if "port_fdi" not in _cache:
        if not os.path.exists(PORT_FDI_SO):
            build()
        o = Oracle(PORT_FDI_SO, "oracle_")
        o.set_gp19_table(_synthetic_gp19())
        _cache["port_fdi"] = o
    return _cache["port_fdi"]


def ref():
    """The reference compiled from its own headers, or None where absent."""
    if "ref" not in _cache:
        _cache["ref"] = Oracle(REF_SO, "ref_") if os.path.exists(REF_SO) else None
    return _cache["ref"]


def ref_native():
    """The reference's optimised build for timing (``-O3``, native CPU,
    OpenMP), compiled on first use from the checkout or its staged copy; None
    where neither exists or the compiler fails."""
    if "ref_native" not in _cache:
        from . import build_ref  # noqa: WPS433
        path = build_ref.build_native()
        _cache["ref_native"] = Oracle(path, "ref_") if path else None
    return _cache["ref_native"]


def _synthetic_gp19():
    import importlib.util
    path = os.path.join(os.path.dirname(HERE), "bns_nurates_gb300", "gp19_synthetic.py")
    spec = importlib.util.spec_from_file_location("gp19_synthetic", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.table()
