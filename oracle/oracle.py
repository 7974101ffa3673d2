"""ctypes bindings of the CPU oracle (TEST INFRASTRUCTURE ONLY).

Only the tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` import this module, and only as the checker / the timed CPU
restatement of the reference.  ``upcg_oracle.h`` states what it is pinned
to: the reference's own src/UpcCrossSection.cpp compiled here against
stand-in GSL / ROOT headers (bit-exact), and scipy for the primitives.
"""
import ctypes as C
import os

import numpy as np

from . import build as _build

_lib = None


def lib():
    global _lib
    if _lib is None:
        so = _build.build_oracle()
        L = C.CDLL(so)
        d, i, p = C.c_double, C.c_int, C.c_void_p
        dp = C.POINTER(C.c_double)
        ip = C.POINTER(C.c_int)
        L.uo_create.restype = p
        L.uo_destroy.argtypes = [p]
        L.uo_set_param.argtypes = [p, C.c_char_p, C.c_char_p]
        L.uo_set_num_threads.argtypes = [p, i]
        L.uo_init_tables.argtypes = [p]
        L.uo_grid.argtypes = [p, dp, dp, ip, dp, dp, ip, dp, dp, ip]
        L.uo_rho0.argtypes = [p]; L.uo_rho0.restype = d
        L.uo_gamma.argtypes = [p]; L.uo_gamma.restype = d
        L.uo_bessel_k01.argtypes = [d, dp, dp]
        L.uo_bessel_k1_as.argtypes = [d]; L.uo_bessel_k1_as.restype = d
        L.uo_simpson.argtypes = [i, dp, d]; L.uo_simpson.restype = d
        L.uo_qags_test.argtypes = [i, d, d, d, d, d, d, i, dp, dp, ip, ip]
        L.uo_spline_natural.argtypes = [i, dp, dp, i, dp, dp]
        for n in ("uo_flux_point",):
            getattr(L, n).argtypes = [p, d, d]; getattr(L, n).restype = d
        L.uo_flux_form.argtypes = [p, d, d, ip, ip, ip]; L.uo_flux_form.restype = d
        for n in ("uo_form_factor", "uo_form_factor_spline", "uo_gaa", "uo_breakup_spline"):
            getattr(L, n).argtypes = [p, d]; getattr(L, n).restype = d
        L.uo_breakup_prob.argtypes = [p, d, i]; L.uo_breakup_prob.restype = d
        L.uo_two_photon_lumi.argtypes = [p, d, d]; L.uo_two_photon_lumi.restype = d
        L.uo_two_photon_lumi_pol.argtypes = [p, d, d, dp, dp]
        L.uo_cs_m.argtypes = [p, d, i]; L.uo_cs_m.restype = d
        L.uo_photon_flux.argtypes = [p, d, d]; L.uo_photon_flux.restype = d
        L.uo_vm_cs_y.argtypes = [p, d]; L.uo_vm_cs_y.restype = d
        L.uo_nuc_cs_y.argtypes = [p, p, p, dp]
        L.uo_cs_zm.argtypes = [p, d, d, i]; L.uo_cs_zm.restype = d
        L.uo_lumi_table.argtypes = [p, p, p, i, i]
        L.uo_cs_zm_table.argtypes = [p, i, p]
        L.uo_nuc_cs_ym.argtypes = [p, p, p, p, p, dp]
        L.uo_generate.argtypes = [p, p, p, p, C.c_int64, C.c_uint64, p,
                                  C.POINTER(C.c_int64), p]
        L.uo_sampler_bin.argtypes = [i, d, d, d]; L.uo_sampler_bin.restype = i
        _lib = L
    return _lib


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


class Oracle:
    """One generator configuration (UpcGenerator + UpcCrossSection state)."""

    def __init__(self, params=None, threads=None):
        self.L = lib()
        self.h = self.L.uo_create()
        self.set_threads(threads or os.cpu_count() or 1)
        for k, v in (params or {}).items():
            self.set_param(k, v)
        self._init = False

    def __del__(self):
        try:
            self.L.uo_destroy(self.h)
        except Exception:
            pass

    def set_threads(self, n):
        self.L.uo_set_num_threads(self.h, int(n))

    def set_param(self, key, value):
        rc = self.L.uo_set_param(self.h, str(key).encode(), str(value).encode())
        if rc < 0:
            raise ValueError(f"bad value for {key}: {value}")
        return rc

    def init_tables(self):
        rc = self.L.uo_init_tables(self.h)
        if rc != 0:
            raise RuntimeError(f"uo_init_tables failed: {rc}")
        self._init = True

    def grid(self):
        v = [C.c_double() for _ in range(6)]
        n = [C.c_int() for _ in range(3)]
        self.L.uo_grid(self.h, C.byref(v[0]), C.byref(v[1]), C.byref(n[0]),
                       C.byref(v[2]), C.byref(v[3]), C.byref(n[1]),
                       C.byref(v[4]), C.byref(v[5]), C.byref(n[2]))
        return dict(mmin=v[0].value, mmax=v[1].value, nm=n[0].value,
                    ymin=v[2].value, ymax=v[3].value, ny=n[1].value,
                    zmin=v[4].value, zmax=v[5].value, nz=n[2].value)

    def rho0(self):
        return self.L.uo_rho0(self.h)

    def gamma(self):
        return self.L.uo_gamma(self.h)

    def flux_point(self, b, k):
        return self.L.uo_flux_point(self.h, b, k)

    def flux_form(self, b, k, info=False):
        st, ne, ni = C.c_int(), C.c_int(), C.c_int()
        v = self.L.uo_flux_form(self.h, b, k, C.byref(st), C.byref(ne), C.byref(ni))
        return (v, st.value, ne.value, ni.value) if info else v

    def form_factor(self, q2):
        return self.L.uo_form_factor(self.h, q2)

    def form_factor_spline(self, q2):
        return self.L.uo_form_factor_spline(self.h, q2)

    def gaa(self, b):
        return self.L.uo_gaa(self.h, b)

    def breakup_prob(self, b, mode):
        return self.L.uo_breakup_prob(self.h, b, mode)

    def breakup_spline(self, b):
        return self.L.uo_breakup_spline(self.h, b)

    def two_photon_lumi(self, m, y):
        return self.L.uo_two_photon_lumi(self.h, m, y)

    def two_photon_lumi_pol(self, m, y):
        s, p = C.c_double(), C.c_double()
        self.L.uo_two_photon_lumi_pol(self.h, m, y, C.byref(s), C.byref(p))
        return s.value, p.value

    def cs_m(self, m, flag=0):
        return self.L.uo_cs_m(self.h, m, flag)

    def photon_flux(self, m, y):
        """calcPhotonFlux (src/UpcCrossSection.cpp:700-722)."""
        return self.L.uo_photon_flux(self.h, m, y)

    def vm_cs_y(self, y):
        """UpcPhotoNuclearVM::calcCrossSectionY in the impulse approximation."""
        return self.L.uo_vm_cs_y(self.h, y)

    def nuc_cs_y(self):
        """calcNucCrossSectionY: (dsigma/dy [ny], emitter ratio [ny], sigma_tot)."""
        ny = self.grid()["ny"]
        cs, ratio, tot = np.zeros(ny), np.zeros(ny), C.c_double()
        if self.L.uo_nuc_cs_y(self.h, _ptr(cs), _ptr(ratio), C.byref(tot)) != 0:
            raise RuntimeError("uo_nuc_cs_y: not a vector-meson configuration")
        return cs, ratio, tot.value

    def cs_zm(self, z, m, flag=0):
        return self.L.uo_cs_zm(self.h, z, m, flag)

    def lumi_table(self, im_lo=0, im_hi=None, polarized=False):
        g = self.grid()
        im_hi = g["nm"] if im_hi is None else im_hi
        out = np.zeros((im_hi - im_lo, g["ny"]))
        out2 = np.zeros_like(out) if polarized else None
        rc = self.L.uo_lumi_table(self.h, _ptr(out), _ptr(out2), im_lo, im_hi)
        if rc != 0:
            raise RuntimeError("lumi_table failed")
        return (out, out2) if polarized else out

    def cs_zm_table(self, flag=0):
        g = self.grid()
        out = np.zeros((g["nm"], g["nz"]))
        self.L.uo_cs_zm_table(self.h, flag, _ptr(out))
        return out

    def nuc_cs_ym(self, lumi, lumi2=None):
        g = self.grid()
        cs = np.zeros((g["ny"], g["nm"]))
        ratio = np.zeros_like(cs) if lumi2 is not None else None
        tot = C.c_double()
        lumi = np.ascontiguousarray(lumi, dtype=np.float64)
        self.L.uo_nuc_cs_ym(self.h, _ptr(lumi), _ptr(lumi2), _ptr(cs), _ptr(ratio), C.byref(tot))
        return cs, tot.value, ratio

    def generate(self, cs_ym, cs_zm, n, seed, ratio=None):
        """Events; polarized: cs_zm = (scalar [nm][nz], pseudoscalar [nm][nz])
        stacked, ratio = nuccs_s / nuccs_p [ny][nm] from nuc_cs_ym (the reference's threshold)."""
        rec = np.zeros((n, 12))
        mbin = np.zeros(n, dtype=np.int32)
        rej = C.c_int64()
        cs_ym = np.ascontiguousarray(cs_ym, dtype=np.float64)
        cs_zm = np.ascontiguousarray(cs_zm, dtype=np.float64)
        rt = np.ascontiguousarray(ratio, dtype=np.float64) if ratio is not None else None
        rc = self.L.uo_generate(self.h, _ptr(cs_ym), _ptr(cs_zm), _ptr(rt) if rt is not None else None,
                                n, seed, _ptr(rec), C.byref(rej), _ptr(mbin))
        if rc != 0:
            raise RuntimeError(f"uo_generate failed: {rc}")
        return rec, rej.value, mbin


def bessel_k01(x):
    k0, k1 = C.c_double(), C.c_double()
    lib().uo_bessel_k01(x, C.byref(k0), C.byref(k1))
    return k0.value, k1.value


def bessel_k1_as(x):
    return lib().uo_bessel_k1_as(x)


def simpson(v, h):
    v = np.ascontiguousarray(v, dtype=np.float64)
    return lib().uo_simpson(len(v), v.ctypes.data_as(C.POINTER(C.c_double)), h)


def qags_test(fid, p0, p1, a, b, epsabs, epsrel, limit=1000):
    r, e, ne, ni = C.c_double(), C.c_double(), C.c_int(), C.c_int()
    st = lib().uo_qags_test(fid, p0, p1, a, b, epsabs, epsrel, limit, C.byref(r), C.byref(e),
                            C.byref(ne), C.byref(ni))
    return r.value, e.value, ne.value, ni.value, st


def spline_natural(x, y, xe):
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.ascontiguousarray(y, dtype=np.float64)
    xe = np.ascontiguousarray(xe, dtype=np.float64)
    ye = np.zeros_like(xe)
    dp = C.POINTER(C.c_double)
    lib().uo_spline_natural(len(x), x.ctypes.data_as(dp), y.ctypes.data_as(dp), len(xe),
                            xe.ctypes.data_as(dp), ye.ctypes.data_as(dp))
    return ye


def sampler_bin(nbins, lo, hi, x):
    return lib().uo_sampler_bin(nbins, lo, hi, x)


_ref_cs = None


def ref_cs_lib():
    """The reference's own UpcCrossSection (src/UpcCrossSection.cpp compiled
    against oracle/refshim/), or None when the reference sources are absent."""
    global _ref_cs
    if _ref_cs is None:
        so = _build.build_ref_cs()
        if so is None:
            return None
        L = C.CDLL(so)
        d, i = C.c_double, C.c_int
        L.uref_cs_init.argtypes = [i, i, d, d, d, i, i, i, d, d, d, d, i, d, d, i, i]
        L.uref_cs_init.restype = i
        for name, args in (("uref_cs_flux_point", [d, d]), ("uref_cs_flux_form", [d, d]),
                           ("uref_cs_form_factor", [d]), ("uref_cs_breakup_prob", [d, i]),
                           ("uref_cs_gaa_spline", [d]), ("uref_cs_breakup_spline", [d]),
                           ("uref_cs_lumi", [d, d]), ("uref_cs_photon_flux", [d, d]),
                           ("uref_cs_rho0", [])):
            f = getattr(L, name)
            f.argtypes = args
            f.restype = d
        L.uref_cs_lumi_pol.argtypes = [d, d, C.POINTER(d), C.POINTER(d)]
        L.uref_cs_lumi_pol.restype = None
        _ref_cs = L
    return _ref_cs


class RefCrossSection:
    """One configuration of the reference's own UpcCrossSection:
    UpcCrossSection::init without the luminosity file, then its member
    functions point by point.  Like the reference, one configuration per
    process: its nucleus and splines are globals, and calcBreakupProb builds
    its photo-neutron tables once per process, for the Lorentz factor of its
    first call (src/UpcCrossSection.cpp:774-898) -- use a fresh process for
    each configuration."""

    def __init__(self, params):
        L = ref_cs_lib()
        if L is None:
            raise RuntimeError("reference sources not present")
        p = dict({"NUCLEUS_Z": 82, "NUCLEUS_A": 208, "WS_R": 6.68, "WS_A": 0.447, "SQRTS": 5020,
                  "FLUX_POINT": 1, "BREAKUP_MODE": 1, "PROC_ID": 15, "ALP_MASS": 1.0,
                  "ALP_WIDTH": 0.01, "MMIN": 3.56, "MMAX": 50, "BINS_M": 1001, "YMIN": -6,
                  "YMAX": 6, "BINS_Y": 121, "USE_POLARIZED_CS": 0}, **params)
        self.L = L
        L.uref_cs_init(int(p["NUCLEUS_Z"]), int(p["NUCLEUS_A"]), float(p["WS_R"]),
                       float(p["WS_A"]), float(p["SQRTS"]), int(p["FLUX_POINT"]),
                       int(p["BREAKUP_MODE"]), int(p["PROC_ID"]), float(p["ALP_MASS"]),
                       float(p["ALP_WIDTH"]), float(p["MMIN"]), float(p["MMAX"]),
                       int(p["BINS_M"]), float(p["YMIN"]), float(p["YMAX"]), int(p["BINS_Y"]),
                       int(p["USE_POLARIZED_CS"]))

    def rho0(self):
        return self.L.uref_cs_rho0()

    def flux_point(self, b, k):
        return self.L.uref_cs_flux_point(b, k)

    def flux_form(self, b, k):
        return self.L.uref_cs_flux_form(b, k)

    def form_factor(self, q2):
        return self.L.uref_cs_form_factor(q2)

    def breakup_prob(self, b, mode):
        return self.L.uref_cs_breakup_prob(b, mode)

    def gaa_spline(self, b):
        return self.L.uref_cs_gaa_spline(b)

    def breakup_spline(self, b):
        return self.L.uref_cs_breakup_spline(b)

    def two_photon_lumi(self, m, y):
        return self.L.uref_cs_lumi(m, y)

    def two_photon_lumi_pol(self, m, y):
        s, q = C.c_double(), C.c_double()
        self.L.uref_cs_lumi_pol(m, y, C.byref(s), C.byref(q))
        return s.value, q.value

    def photon_flux(self, m, y):
        return self.L.uref_cs_photon_flux(m, y)


_ref = None


def ref_lib():
    """The reference's own elementary cross sections (None if not buildable)."""
    global _ref
    if _ref is None:
        so = _build.build_ref()
        if so is None:
            return None
        L = C.CDLL(so)
        d, i = C.c_double, C.c_int
        L.uref_dilep_cs_m.argtypes = [i, d, d, i]; L.uref_dilep_cs_m.restype = d
        L.uref_dilep_cs_zm.argtypes = [i, d, d, d, i]; L.uref_dilep_cs_zm.restype = d
        L.uref_dilep_mass.argtypes = [i]; L.uref_dilep_mass.restype = d
        L.uref_alp_cs_m.argtypes = [d, d, d]; L.uref_alp_cs_m.restype = d
        _ref = L
    return _ref
