"""upcgen-gb300: GB300 (sm_103a) implementation of upcgen's two-photon
luminosity, nuclear cross-section and (m, y, z) event-sampling path.

Python mirror of the reference's ``UpcGenerator`` / ``UpcCrossSection`` API
(include/UpcGenerator.h:55-128, include/UpcCrossSection.h:65-240) over the C ABI
of ``include/upcgen_gb300.h``, implemented by ``libupcgen_gb300.so``.  There is
no CPU implementation behind it: if the CUDA library is absent or no GPU is
visible, constructing a generator raises.
"""
import ctypes as C
import os

import numpy as np

__all__ = ["UpcGenerator", "UpcCrossSection", "UpcgError", "EVENT_DTYPE", "library_path",
           "load_library", "philox"]

_HERE = os.path.dirname(os.path.abspath(__file__))
library_path = os.path.join(_HERE, "libupcgen_gb300.so")

EVENT_DTYPE = np.dtype([("m", "<f4"), ("y", "<f4"), ("z", "<f4"), ("sign", "<f4"),
                        ("p0", "<f4", (4,)), ("p1", "<f4", (4,))])
assert EVENT_DTYPE.itemsize == 48

# every symbol include/upcgen_gb300.h declares
ABI_SYMBOLS = [
    "upcg_create", "upcg_destroy", "upcg_set_parameter", "upcg_config_from_file",
    "upcg_set_collision_system", "upcg_set_seed", "upcg_set_num_threads",
    "upcg_set_debug_level", "upcg_set_lumi_file_directory", "upcg_set_lumi_cache", "upcg_lumi_cache_file",
    "upcg_particles_per_event", "upcg_event_particles_device", "upcg_format_hepmc3",
    "upcg_write_events", "upcg_run_events", "upcg_sampler_bins", "upcg_photon_flux", "upcg_vm_cross_section_y", "upcg_nuc_cs_y",
    "upcg_decay_pdg", "upcg_contract_rows", "upcg_contract_work",
    "upcg_set_stream", "upcg_set_lumi_method", "upcg_init", "upcg_compute_nucl_xsection",
    "upcg_tot_nucl_x", "upcg_fid_nucl_x", "upcg_get_grid", "upcg_lumi_table",
    "upcg_lumi_table_device", "upcg_nuc_cs_ym", "upcg_cs_zm_table", "upcg_flux_point",
    "upcg_flux_form", "upcg_form_factor", "upcg_breakup_prob", "upcg_eval_spline",
    "upcg_two_photon_lumi", "upcg_cs_m", "upcg_generate_events",
    "upcg_generate_events_device", "upcg_generate_event", "upcg_philox",
    "upcg_host_alloc", "upcg_host_free",
    "upcg_last_timings", "upcg_qags_stats", "upcg_last_error", "upcg_version",
    "upcg_selftest_contract", "upcg_fast_flux_table", "upcg_kernel_launches",
    "upcg_flux_form_device_noalloc", "upcg_copy_bytes", "upcg_particle_pdg",
    "upcg_set_row_range", "upcg_set_lumi_table", "upcg_set_lumi_table_device", "upcg_set_candidate_offset",
    "upcg_get_candidate_offset", "upcg_event_output_config",
    "upcg_mlp_create", "upcg_mlp_destroy", "upcg_mlp_box", "upcg_mlp_make_data",
    "upcg_mlp_get_data", "upcg_mlp_train", "upcg_mlp_gradients", "upcg_mlp_params",
    "upcg_mlp_set_params", "upcg_mlp_predict", "upcg_mlp_timings", "upcg_set_flux_surrogate",
    "upcg_surrogate_rows", "upcg_scan_create", "upcg_scan_run", "upcg_scan_info",
    "upcg_scan_destroy",
]


class UpcgError(RuntimeError):
    pass


_lib = None


def load_library(path=None):
    """Load (never build) the CUDA library; raises if it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or library_path
    if not os.path.exists(path):
        raise UpcgError(f"{path} is missing: run `python -c 'import __graft_entry__ as g; g.build()'`")
    L = C.CDLL(path)
    vp, cp, i, d, sz = C.c_void_p, C.c_char_p, C.c_int, C.c_double, C.c_size_t
    i64, u64 = C.c_int64, C.c_uint64
    dp = C.POINTER(C.c_double)
    sig = {
        "upcg_create": [C.POINTER(vp)], "upcg_destroy": [vp],
        "upcg_set_parameter": [vp, cp, cp], "upcg_config_from_file": [vp, cp],
        "upcg_set_collision_system": [vp, C.c_float, i, i], "upcg_set_seed": [vp, C.c_long],
        "upcg_set_num_threads": [vp, i], "upcg_set_debug_level": [vp, i],
        "upcg_set_lumi_file_directory": [vp, cp], "upcg_set_lumi_cache": [vp, i],
        "upcg_lumi_cache_file": [vp, cp, C.c_size_t, C.POINTER(C.c_int)],
        "upcg_particles_per_event": [vp, C.POINTER(i)],
        "upcg_event_particles_device": [vp, vp, i64, i64, vp],
        "upcg_format_hepmc3": [vp, vp, i64, i64, vp, sz, C.POINTER(sz)],
        "upcg_write_events": [vp, cp, i64, i, i, C.POINTER(i64)],
        "upcg_run_events": [vp, i64, C.POINTER(i64)],
        "upcg_sampler_bins": [vp, vp, sz, i, vp],
        "upcg_photon_flux": [vp, vp, vp, vp, sz], "upcg_vm_cross_section_y": [vp, vp, vp, sz],
        "upcg_nuc_cs_y": [vp, vp, vp, sz, dp], "upcg_decay_pdg": [vp, C.POINTER(i)],
        "upcg_contract_rows": [vp, C.POINTER(i64)],
        "upcg_contract_work": [vp, C.POINTER(i64), C.POINTER(i64)],
        "upcg_set_stream": [vp, vp], "upcg_set_lumi_method": [vp, i], "upcg_init": [vp],
        "upcg_compute_nucl_xsection": [vp], "upcg_tot_nucl_x": [vp, dp],
        "upcg_fid_nucl_x": [vp, dp],
        "upcg_get_grid": [vp, dp, dp, C.POINTER(i), dp, dp, C.POINTER(i), dp, dp, C.POINTER(i)],
        "upcg_lumi_table": [vp, vp, sz, vp], "upcg_lumi_table_device": [vp, vp, vp],
        "upcg_nuc_cs_ym": [vp, vp, sz, dp], "upcg_cs_zm_table": [vp, i, vp, sz],
        "upcg_flux_point": [vp, vp, vp, vp, sz], "upcg_flux_form": [vp, vp, vp, vp, sz],
        "upcg_form_factor": [vp, vp, vp, sz], "upcg_breakup_prob": [vp, vp, i, vp, sz],
        "upcg_eval_spline": [vp, i, vp, vp, sz], "upcg_two_photon_lumi": [vp, vp, vp, vp, vp, sz],
        "upcg_cs_m": [vp, vp, i, vp, sz], "upcg_generate_events": [vp, i64, vp, vp, C.POINTER(i64)],
        "upcg_generate_events_device": [vp, i64, vp, vp, C.POINTER(i64)],
        "upcg_generate_event": [vp, vp, C.POINTER(i)], "upcg_philox": [u64, u64, sz, vp],
        "upcg_host_alloc": [sz, C.POINTER(vp)], "upcg_host_free": [vp],
        "upcg_last_timings": [vp, dp, sz],
        "upcg_qags_stats": [vp, C.POINTER(u64), C.POINTER(u64), C.POINTER(u64)],
        "upcg_last_error": [], "upcg_version": [],
        "upcg_selftest_contract": [i, i, u64, dp, dp],
        "upcg_fast_flux_table": [vp, vp, sz, vp],
        "upcg_kernel_launches": [C.POINTER(u64)],
        "upcg_flux_form_device_noalloc": [vp, vp, vp, vp, sz, vp],
        "upcg_copy_bytes": [C.POINTER(u64), C.POINTER(u64)],
        "upcg_particle_pdg": [vp, C.POINTER(i), C.POINTER(i)],
        "upcg_set_row_range": [vp, i, i], "upcg_set_lumi_table": [vp, vp, sz, vp],
        "upcg_set_lumi_table_device": [vp, vp, sz, vp],
        "upcg_set_candidate_offset": [vp, u64],
        "upcg_get_candidate_offset": [vp, C.POINTER(u64)],
        "upcg_event_output_config": [vp, C.POINTER(i64), C.POINTER(i), C.POINTER(i)],
        "upcg_mlp_create": [C.POINTER(vp), u64], "upcg_mlp_destroy": [vp],
        "upcg_mlp_box": [vp, vp, sz], "upcg_mlp_make_data": [vp, i64, u64],
        "upcg_mlp_get_data": [vp, i64, i64, vp, vp, vp],
        "upcg_mlp_train": [vp, i, i, C.c_float, dp],
        "upcg_mlp_gradients": [vp, vp, vp, vp, i, vp, sz, dp],
        "upcg_mlp_params": [vp, vp, sz], "upcg_mlp_set_params": [vp, vp, sz],
        "upcg_mlp_predict": [vp, vp, i, vp], "upcg_mlp_timings": [vp, dp, dp],
        "upcg_set_flux_surrogate": [vp, vp], "upcg_surrogate_rows": [vp, C.POINTER(i)],
        "upcg_scan_create": [C.POINTER(vp), C.POINTER(vp), i], "upcg_scan_run": [vp, dp],
        "upcg_scan_info": [vp, C.POINTER(i), C.POINTER(i), C.POINTER(i), dp],
        "upcg_scan_destroy": [vp],
    }
    for name, args in sig.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = cp if name in ("upcg_last_error", "upcg_version") else i
    _lib = L
    return L


def _check(rc):
    if rc != 0:
        raise UpcgError(f"status {rc}: {_lib.upcg_last_error().decode(errors='replace')}")
    return rc


def _arr(x):
    return np.ascontiguousarray(x, dtype=np.float64)


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def _out_array(out, shape, dtype=np.float64):
    """A fresh zeroed array, or the caller's after checking it fits."""
    if out is None:
        return np.zeros(shape, dtype=dtype)
    if out.dtype != dtype or out.shape != tuple(shape) or not out.flags.c_contiguous \
            or not out.flags.writeable:
        raise ValueError(f"out must be a writeable C-contiguous {np.dtype(dtype)} array of shape {tuple(shape)}")
    return out


def selftest_contract(ncells, P, seed=1):
    """Tensor-core contraction vs FP64 on random data: (max rel err, ms)."""
    L = load_library()
    e, t = C.c_double(), C.c_double()
    _check(L.upcg_selftest_contract(int(ncells), int(P), int(seed), C.byref(e), C.byref(t)))
    return e.value, t.value


def kernel_launches():
    """Kernels the library has launched in this process so far."""
    L = load_library()
    n = C.c_uint64()
    _check(L.upcg_kernel_launches(C.byref(n)))
    return n.value


def copy_bytes():
    """(host-to-device, device-to-host) bytes the library has copied so far."""
    L = load_library()
    a, b = C.c_uint64(), C.c_uint64()
    _check(L.upcg_copy_bytes(C.byref(a), C.byref(b)))
    return a.value, b.value


class _PinnedBlock:
    """Page-locked host bytes from upcg_host_alloc, freed with the last view."""

    def __init__(self, nbytes):
        self._L = load_library()
        self.ptr = C.c_void_p()
        _check(self._L.upcg_host_alloc(int(nbytes), C.byref(self.ptr)))
        self.nbytes = int(nbytes)

    def __del__(self):
        if getattr(self, "ptr", None) and self.ptr.value:
            self._L.upcg_host_free(self.ptr)
            self.ptr = C.c_void_p()


def pinned_array(shape, dtype):
    """A numpy array in page-locked host memory (e.g. the out= buffer of
    generateEvents); the memory lives as long as the array or a view of it."""
    dtype = np.dtype(dtype)
    n = int(np.prod(shape))
    blk = _PinnedBlock(max(n * dtype.itemsize, 1))
    buf = (C.c_char * blk.nbytes).from_address(blk.ptr.value)
    buf._upcg_block = blk  # keeps the block alive while numpy holds the buffer
    return np.frombuffer(buf, dtype=dtype, count=n).reshape(shape)


def philox(seed, counter0, n):
    """Philox4x32-10 words of the event stream, computed on the GPU."""
    L = load_library()
    out = np.zeros((n, 4), dtype=np.uint32)
    _check(L.upcg_philox(seed, counter0, n, _p(out)))
    return out


class FluxSurrogate:
    """The learned flux surrogate (upcg_mlp_*): y = ln(Q_ff / Q_pt) from
    normalised (ln w, ln b, R, a, ln g)."""

    N_PARAMS = 5 * 128 + 128 + 3 * (128 * 128 + 128) + 128 + 1

    def __init__(self, seed=1):
        self._L = load_library()
        self._h = C.c_void_p()
        _check(self._L.upcg_mlp_create(C.byref(self._h), int(seed)))

    def __del__(self):
        if getattr(self, "_h", None) and self._h.value:
            self._L.upcg_mlp_destroy(self._h)
            self._h = C.c_void_p()

    def box(self):
        b = np.zeros(10, dtype=np.float32)
        _check(self._L.upcg_mlp_box(self._h, _p(b), 10))
        keys = ["lw_lo", "lw_hi", "bf_lo", "lb_hi", "R_lo", "R_hi", "a_lo", "a_hi", "g_lo", "g_hi"]
        return dict(zip(keys, (float(v) for v in b)))

    def normalise(self, w, b, R, a, g):
        bx = self.box()
        u = np.empty((np.size(w), 5), dtype=np.float32)
        lb_lo = np.log(bx["bf_lo"] * bx["R_lo"])
        u[:, 0] = 2 * (np.log(w) - bx["lw_lo"]) / (bx["lw_hi"] - bx["lw_lo"]) - 1
        u[:, 1] = 2 * (np.log(b) - lb_lo) / (bx["lb_hi"] - lb_lo) - 1
        u[:, 2] = 2 * (np.asarray(R) - bx["R_lo"]) / (bx["R_hi"] - bx["R_lo"]) - 1
        u[:, 3] = 2 * (np.asarray(a) - bx["a_lo"]) / (bx["a_hi"] - bx["a_lo"]) - 1
        u[:, 4] = 2 * (np.log(g) - np.log(bx["g_lo"])) / (np.log(bx["g_hi"]) - np.log(bx["g_lo"])) - 1
        return u

    def make_data(self, n, seed=1):
        _check(self._L.upcg_mlp_make_data(self._h, int(n), int(seed)))

    def data(self, i0, n):
        x = np.zeros((n, 5), dtype=np.float32)
        y = np.zeros(n, dtype=np.float32)
        w = np.zeros(n, dtype=np.float32)
        _check(self._L.upcg_mlp_get_data(self._h, int(i0), int(n), _p(x), _p(y), _p(w)))
        return x, y, w

    def train(self, epochs, batch=4096, lr=2e-3):
        loss = C.c_double()
        _check(self._L.upcg_mlp_train(self._h, int(epochs), int(batch), C.c_float(lr), C.byref(loss)))
        return loss.value

    @staticmethod
    def _inputs(x, n=None):
        """(n, 5) float32 network inputs; the library reads 5 floats per point."""
        x = np.ascontiguousarray(x, dtype=np.float32)
        if x.ndim != 2 or x.shape[1] != 5 or (n is not None and x.shape[0] != n):
            raise ValueError(f"inputs must have shape ({'n' if n is None else n}, 5), got {x.shape}")
        return x

    def gradients(self, x, y, w):
        y = np.ascontiguousarray(y, dtype=np.float32).ravel()
        w = np.ascontiguousarray(w, dtype=np.float32).ravel()
        if w.size != y.size:
            raise ValueError(f"{y.size} labels but {w.size} weights")
        x = self._inputs(x, y.size)
        g = np.zeros(self.N_PARAMS, dtype=np.float32)
        loss = C.c_double()
        _check(self._L.upcg_mlp_gradients(self._h, _p(x), _p(y), _p(w), len(y), _p(g), g.size,
                                          C.byref(loss)))
        return g, loss.value

    def params(self):
        p = np.zeros(self.N_PARAMS, dtype=np.float32)
        _check(self._L.upcg_mlp_params(self._h, _p(p), p.size))
        return p

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        _check(self._L.upcg_mlp_set_params(self._h, _p(p), p.size))

    def predict(self, x):
        x = self._inputs(x)
        y = np.zeros(len(x), dtype=np.float32)
        _check(self._L.upcg_mlp_predict(self._h, _p(x), len(x), _p(y)))
        return y

    def timings(self):
        a, b = C.c_double(), C.c_double()
        _check(self._L.upcg_mlp_timings(self._h, C.byref(a), C.byref(b)))
        return {"labels_ms": a.value, "train_ms": b.value}


class Scan:
    """Batched table build of several configurations (upcg_scan_*): one
    persistent tensor-core contraction over all of them, replayed from a
    captured CUDA graph."""

    def __init__(self, generators):
        self._L = load_library()
        self.generators = list(generators)  # kept alive with the scan
        arr = (C.c_void_p * len(self.generators))(*[g._h.value for g in self.generators])
        self._h = C.c_void_p()
        _check(self._L.upcg_scan_create(C.byref(self._h), arr, len(self.generators)))

    def run(self):
        ms = C.c_double()
        _check(self._L.upcg_scan_run(self._h, C.byref(ms)))
        return ms.value

    def info(self):
        n, sh, rows, st = C.c_int(), C.c_int(), C.c_int(), C.c_double()
        _check(self._L.upcg_scan_info(self._h, C.byref(n), C.byref(sh), C.byref(rows), C.byref(st)))
        return {"items": n.value, "shape": ["256x2", "128x3"][sh.value], "rows": rows.value,
                "setup_ms": st.value}

    def __del__(self):
        if getattr(self, "_h", None) and self._h.value:
            self._L.upcg_scan_destroy(self._h)
            self._h = C.c_void_p()


class UpcCrossSection:
    """Batched views of the UpcCrossSection methods of a generator."""

    def __init__(self, gen):
        self._g = gen

    def _pts(self, fn, *arrays, extra=()):
        arrays = [_arr(a) for a in arrays]
        out = np.zeros_like(arrays[0])
        _check(fn(*([self._g._h] + [_p(a) for a in arrays] + list(extra) + [_p(out), out.size])))
        return out

    def fluxPoint(self, b, k):  # src/UpcCrossSection.cpp:166-178
        b, k = np.broadcast_arrays(_arr(b), _arr(k))
        return self._pts(self._g._L.upcg_flux_point, b, k)

    def fluxForm(self, b, k):  # src/UpcCrossSection.cpp:194-218
        b, k = np.broadcast_arrays(_arr(b), _arr(k))
        return self._pts(self._g._L.upcg_flux_form, b, k)

    def fluxFormDeviceNoAlloc(self, b_ptr, k_ptr, out_ptr, n, failures_ptr=None):
        """fluxForm on device buffers (raw device pointers, n doubles each)
        without any device allocation (upcg_flux_form_device_noalloc; no
        counterpart in the reference).  Asynchronous on the generator's stream."""
        _check(self._g._L.upcg_flux_form_device_noalloc(
            self._g._h, C.c_void_p(b_ptr), C.c_void_p(k_ptr), C.c_void_p(out_ptr), int(n),
            C.c_void_p(failures_ptr) if failures_ptr else None))

    def calcFormFac(self, q2):  # src/UpcCrossSection.cpp:436-445
        return self._pts(self._g._L.upcg_form_factor, q2)

    def calcBreakupProb(self, b, mode):  # src/UpcCrossSection.cpp:752-1019
        b = _arr(b)
        out = np.zeros_like(b)
        _check(self._g._L.upcg_breakup_prob(self._g._h, _p(b), int(mode), _p(out), out.size))
        return out

    def spline(self, which, x):
        """Tabulated splines: 'gaa', 'breakup' or 'formfac'."""
        idx = {"gaa": 0, "breakup": 1, "formfac": 2}[which]
        x = _arr(x)
        out = np.zeros_like(x)
        _check(self._g._L.upcg_eval_spline(self._g._h, idx, _p(x), _p(out), out.size))
        return out

    def calcTwoPhotonLumi(self, M, Y):  # src/UpcCrossSection.cpp:221-271
        M, Y = np.broadcast_arrays(_arr(M), _arr(Y))
        M, Y = _arr(M), _arr(Y)
        out = np.zeros_like(M)
        _check(self._g._L.upcg_two_photon_lumi(self._g._h, _p(M), _p(Y), _p(out), None, out.size))
        return out

    def calcTwoPhotonLumiPol(self, M, Y):  # src/UpcCrossSection.cpp:274-335
        M, Y = np.broadcast_arrays(_arr(M), _arr(Y))
        M, Y = _arr(M), _arr(Y)
        s, p = np.zeros_like(M), np.zeros_like(M)
        _check(self._g._L.upcg_two_photon_lumi(self._g._h, _p(M), _p(Y), _p(s), _p(p), s.size))
        return s, p

    def calcCrossSectionM(self, m, flag=0):  # elementary process sigma(m)
        m = _arr(m)
        out = np.zeros_like(m)
        _check(self._g._L.upcg_cs_m(self._g._h, _p(m), int(flag), _p(out), out.size))
        return out

    def fillCrossSectionZM(self, flag=0):  # src/UpcCrossSection.cpp:337-362, [nm][nz]
        return self._g.crossSectionZM(flag)

    def calcNucCrossSectionYM(self, out=None):  # src/UpcCrossSection.cpp:594-698
        """(dsigma [ny][nm] in nb, sigma_tot in mb)."""
        return self._g.nucCSYM(out=out)

    def calcPhotonFlux(self, m, y):  # src/UpcCrossSection.cpp:700-722
        return self._g.calcPhotonFlux(m, y)

    def calcNucCrossSectionY(self):  # src/UpcCrossSection.cpp:724-748
        """(dsigma/dy [ny], emitter ratio [ny], sigma_tot mb) of a vector meson."""
        return self._g.nucCSY()


class UpcGenerator:
    """Mirror of upcgen's UpcGenerator (include/UpcGenerator.h:55-128)."""

    def __init__(self, params=None, lib_path=None):
        self._L = load_library(lib_path)
        h = C.c_void_p()
        _check(self._L.upcg_create(C.byref(h)))
        self._h = h
        self._parfile = "parameters.in"
        self.nucProcessCS = UpcCrossSection(self)
        for k, v in (params or {}).items():
            self.setParameterValue(k, v)

    def __del__(self):
        try:
            if getattr(self, "_h", None):
                self._L.upcg_destroy(self._h)
                self._h = None
        except Exception:
            pass

    # -- configuration
    def setParameterValue(self, parameter, parValue):
        _check(self._L.upcg_set_parameter(self._h, str(parameter).encode(), str(parValue).encode()))

    def setParFile(self, parfilename):
        self._parfile = parfilename

    def configGeneratorFromFile(self):
        _check(self._L.upcg_config_from_file(self._h, self._parfile.encode()))

    def setCollisionSystem(self, sqrts, nucl_z, nucl_a):
        _check(self._L.upcg_set_collision_system(self._h, float(sqrts), int(nucl_z), int(nucl_a)))

    def setSeed(self, seed):
        _check(self._L.upcg_set_seed(self._h, int(seed)))

    def setNumThreads(self, n):
        _check(self._L.upcg_set_num_threads(self._h, int(n)))

    def setDebugLevel(self, level):
        _check(self._L.upcg_set_debug_level(self._h, int(level)))

    def setLumiFileDirectory(self, directory):
        _check(self._L.upcg_set_lumi_file_directory(self._h, str(directory).encode()))

    def setLumiCache(self, enable):
        _check(self._L.upcg_set_lumi_cache(self._h, int(bool(enable))))

    def lumiCacheFile(self):
        """(path of this configuration's cache file, last_hit): last_hit 1 if
        the last init read the table from it, 0 if it computed the table, -1
        if the cache was not used."""
        buf = C.create_string_buffer(4096)
        hit = C.c_int()
        _check(self._L.upcg_lumi_cache_file(self._h, buf, len(buf), C.byref(hit)))
        return buf.value.decode(), hit.value

    def setStream(self, stream_handle):
        _check(self._L.upcg_set_stream(self._h, C.c_void_p(int(stream_handle) if stream_handle else 0)))

    def setLumiMethod(self, method):
        _check(self._L.upcg_set_lumi_method(self._h, {"plain": 0, "fast": 1, "hybrid": 2, "grid": 3, "surrogate": 4,
                                                                 "gather": 5, "fused": 6,
                                                                 "grid-tf32": 7}.get(method, method)))

    # -- sharding over m-rows (upcgen_gb300.shard)
    def setRowRange(self, im0, im1=-1):
        _check(self._L.upcg_set_row_range(self._h, int(im0), int(im1)))

    def setLumiTable(self, table, table2=None):
        t = _arr(table).ravel()
        t2 = _arr(table2).ravel() if table2 is not None else None
        if t2 is not None and t2.size != t.size:
            raise ValueError(f"the two tables differ in size ({t.size}, {t2.size})")
        _check(self._L.upcg_set_lumi_table(self._h, _p(t), t.size, _p(t2) if t2 is not None else None))

    def setLumiTableDevice(self, ptr, n, ptr2=None):
        """Install a full table from device memory (raw device pointers to
        n float64 each; upcg_set_lumi_table_device)."""
        _check(self._L.upcg_set_lumi_table_device(self._h, C.c_void_p(ptr), int(n),
                                                  C.c_void_p(ptr2) if ptr2 else None))

    def lumiTableDevicePtrs(self):
        """(device pointer of the table, of the pseudoscalar table or 0):
        valid until the next init on this generator."""
        a, b = C.c_void_p(), C.c_void_p()
        _check(self._L.upcg_lumi_table_device(self._h, C.byref(a), C.byref(b)))
        return a.value or 0, b.value or 0

    def fastFluxTable(self):
        """The fast form's form-factor flux amplitude table Q[512][256] on
        (ln w, ln b) and its grid (ln w0, h_w, ln b0, h_b)."""
        out = np.zeros((512, 256))
        grid = np.zeros(4)
        _check(self._L.upcg_fast_flux_table(self._h, _p(out), out.size, _p(grid)))
        return out, tuple(grid)

    def setFluxSurrogate(self, surrogate):
        self._surrogate = surrogate  # kept alive with the generator
        _check(self._L.upcg_set_flux_surrogate(self._h, surrogate._h if surrogate else None))

    def surrogateRows(self):
        r = C.c_int()
        _check(self._L.upcg_surrogate_rows(self._h, C.byref(r)))
        return r.value

    def setCandidateOffset(self, counter):
        _check(self._L.upcg_set_candidate_offset(self._h, int(counter)))

    # -- computation
    def init(self):
        _check(self._L.upcg_init(self._h))

    def computeNuclXsection(self):
        _check(self._L.upcg_compute_nucl_xsection(self._h))

    def totNuclX(self):
        v = C.c_double()
        _check(self._L.upcg_tot_nucl_x(self._h, C.byref(v)))
        return v.value

    def fidNuclX(self):
        v = C.c_double()
        _check(self._L.upcg_fid_nucl_x(self._h, C.byref(v)))
        return v.value

    def grid(self):
        v = [C.c_double() for _ in range(6)]
        n = [C.c_int() for _ in range(3)]
        _check(self._L.upcg_get_grid(self._h, C.byref(v[0]), C.byref(v[1]), C.byref(n[0]),
                                     C.byref(v[2]), C.byref(v[3]), C.byref(n[1]),
                                     C.byref(v[4]), C.byref(v[5]), C.byref(n[2])))
        return dict(mmin=v[0].value, mmax=v[1].value, nm=n[0].value, ymin=v[2].value,
                    ymax=v[3].value, ny=n[1].value, zmin=v[4].value, zmax=v[5].value, nz=n[2].value)

    def lumiTable(self, polarized=False, out=None, out2=None):
        """L dm dy [nm][ny] (and the pseudoscalar table when polarized); out /
        out2: a caller's float64 arrays of that shape (pinned_array for the
        fastest copy)."""
        g = self.grid()
        out = _out_array(out, (g["nm"], g["ny"]))
        out2 = _out_array(out2, (g["nm"], g["ny"])) if polarized else None
        _check(self._L.upcg_lumi_table(self._h, _p(out), out.size, _p(out2) if polarized else None))
        return (out, out2) if polarized else out

    def nucCSYM(self, out=None):
        """(dsigma [ny][nm], sigma_tot mb); out: a caller's float64 [ny][nm] array."""
        g = self.grid()
        out = _out_array(out, (g["ny"], g["nm"]))
        tot = C.c_double()
        _check(self._L.upcg_nuc_cs_ym(self._h, _p(out), out.size, C.byref(tot)))
        return out, tot.value

    def crossSectionZM(self, flag=0):
        g = self.grid()
        out = np.zeros((g["nm"], g["nz"]))
        _check(self._L.upcg_cs_zm_table(self._h, int(flag), _p(out), out.size))
        return out

    def generateEvents(self, n, with_mbin=False, out=None):
        """The accepted-event loop; returns (events, rejected[, mbin]).  out:
        a caller's EVENT_DTYPE array of at least n records (pinned_array for
        the fastest copy); the events are its first n."""
        if out is None:
            out = np.zeros(int(n), dtype=EVENT_DTYPE)
        else:
            if out.dtype != EVENT_DTYPE or not out.flags.c_contiguous or out.size < int(n):
                raise ValueError("out must be a C-contiguous EVENT_DTYPE array of at least n records")
            out = out[:int(n)]
        mb = np.zeros(int(n), dtype=np.int32) if with_mbin else None
        rej = C.c_int64()
        _check(self._L.upcg_generate_events(self._h, int(n), _p(out), _p(mb) if with_mbin else None,
                                            C.byref(rej)))
        return (out, rej.value, mb) if with_mbin else (out, rej.value)

    # -- photonuclear path (vector mesons)
    def calcPhotonFlux(self, m, y):
        """UpcCrossSection::calcPhotonFlux at points (m, y)."""
        m, y = np.broadcast_arrays(_arr(m), _arr(y))
        m, y = np.ascontiguousarray(m), np.ascontiguousarray(y)
        out = np.zeros(m.size)
        _check(self._L.upcg_photon_flux(self._h, _p(m), _p(y), _p(out), m.size))
        return out

    def vmCrossSectionY(self, y):
        """UpcPhotoNuclearVM::calcCrossSectionY (impulse approximation)."""
        y = np.ascontiguousarray(_arr(y))
        out = np.zeros(y.size)
        _check(self._L.upcg_vm_cross_section_y(self._h, _p(y), _p(out), y.size))
        return out

    def nucCSY(self):
        """calcNucCrossSectionY: (dsigma/dy [ny], emitter ratio [ny], sigma_tot mb)."""
        ny = self.grid()["ny"]
        cs, ratio, tot = np.zeros(ny), np.zeros(ny), C.c_double()
        _check(self._L.upcg_nuc_cs_y(self._h, _p(cs), _p(ratio), ny, C.byref(tot)))
        return cs, ratio, tot.value

    def contractRows(self):
        """Rows of the last fast-form contraction (cells computed; their mirror
        cells are copies)."""
        n = C.c_int64()
        _check(self._L.upcg_contract_rows(self._h, C.byref(n)))
        return n.value

    def contractWork(self):
        """(rows, multiply-adds per row) of the last fast-form contraction: the
        tiles where the survival kernel minus its constant can be nonzero."""
        n, m = C.c_int64(), C.c_int64()
        _check(self._L.upcg_contract_work(self._h, C.byref(n), C.byref(m)))
        return n.value, m.value

    def decayPDG(self):
        n = C.c_int()
        _check(self._L.upcg_decay_pdg(self._h, C.byref(n)))
        return n.value

    def particlesPerEvent(self):
        n = C.c_int()
        _check(self._L.upcg_particles_per_event(self._h, C.byref(n)))
        return n.value

    def formatHepMC3(self, events, first_event=0):
        """HepMC3 ASCII lines of host event records (no version / listing lines)."""
        ev = np.ascontiguousarray(events, dtype=EVENT_DTYPE)
        n = C.c_size_t()
        rc = self._L.upcg_format_hepmc3(self._h, _p(ev), len(ev), int(first_event), None, 0, C.byref(n))
        if rc not in (0, -7):
            _check(rc)
        buf = C.create_string_buffer(n.value + 1)
        _check(self._L.upcg_format_hepmc3(self._h, _p(ev), len(ev), int(first_event), buf, len(buf),
                                          C.byref(n)))
        return buf.raw[:n.value].decode()

    def eventOutputConfig(self):
        """(NEVENTS, USE_ROOT_OUTPUT, USE_HEPMC_OUTPUT) as configured."""
        n, r, h = C.c_int64(), C.c_int(), C.c_int()
        _check(self._L.upcg_event_output_config(self._h, C.byref(n), C.byref(r), C.byref(h)))
        return n.value, r.value, h.value

    def candidateOffset(self):
        """The Philox counter the next event entry starts at."""
        c = C.c_uint64()
        _check(self._L.upcg_get_candidate_offset(self._h, C.byref(c)))
        return c.value

    def generateEventFiles(self, directory="."):
        """The reference's generateEvents() (src/UpcGenerator.cpp:834-926):
        NEVENTS events to events.hepmc (USE_HEPMC_OUTPUT) and to the particles
        tree's column file events.cols (USE_ROOT_OUTPUT, on unless set to 0;
        particles_to_root.C makes events.root); both files hold the same
        events.  With neither file configured the loop still runs (the events
        are drawn and dropped), so the candidate sequence, the rejected count
        and fidNuclX end where the reference's do.  Returns the rejected
        count."""
        n, use_root, use_hepmc = self.eventOutputConfig()
        if not use_root and not use_hepmc:
            rej = C.c_int64()
            _check(self._L.upcg_run_events(self._h, int(n), C.byref(rej)))
            return rej.value
        c0 = self.candidateOffset()
        rej = None
        if use_hepmc:
            rej = self.writeEvents(os.path.join(directory, "events.hepmc"), n, "hepmc")
        if use_root:
            if use_hepmc:
                self.setCandidateOffset(c0)
            rej = self.writeEvents(os.path.join(directory, "events.cols"), n, "columns")
        return rej

    def writeEvents(self, path, n, format="hepmc", threads=0):
        """generateEvents with file output (HepMC3 ASCII, or the particle
        columns of the reference's ROOT tree); returns the rejected count."""
        fmt = {"hepmc": 0, "columns": 1}.get(format, format)
        rej = C.c_int64()
        _check(self._L.upcg_write_events(self._h, str(path).encode(), int(n), int(fmt), int(threads),
                                         C.byref(rej)))
        return rej.value

    def samplerBins(self, x, axis="m"):
        """The event kernels' getBinY (axis "m") / getBinX (axis "y") of the
        (y, m) sampler on the values x (include/UpcSampler.h:124-134)."""
        x = _arr(x).ravel()
        out = np.zeros(x.size, dtype=np.int32)
        _check(self._L.upcg_sampler_bins(self._h, _p(x), x.size, {"m": 0, "y": 1}[axis], _p(out)))
        return out

    def generateEvent(self):
        """One candidate: (1 or 0, event record), as UpcGenerator::generateEvent."""
        ev = np.zeros(1, dtype=EVENT_DTYPE)
        acc = C.c_int()
        _check(self._L.upcg_generate_event(self._h, _p(ev), C.byref(acc)))
        self._last_record = ev[0]
        return acc.value, ev[0]

    def particlePDG(self):
        """(PDG code of the final state, whether it is charged)."""
        p, q = C.c_int(), C.c_int()
        _check(self._L.upcg_particle_pdg(self._h, C.byref(p), C.byref(q)))
        return p.value, bool(q.value)

    def particlesOf(self, rec):
        """generateEvent's particle lists for one record (src/UpcGenerator.cpp:
        767-812): [(pdg, status, mother, (px, py, pz, e))].  A lepton pair: two
        leptons, status 23, mother 0, opposite charges by the record's sign; an
        ALP or a vector meson: the parent (status 23, momentum = the daughters'
        sum) and its two daughters (status 33, mother 1)."""
        pdg, charged = self.particlePDG()
        a = tuple(float(x) for x in rec["p0"])
        b = tuple(float(x) for x in rec["p1"])
        s1 = 1 if rec["sign"] > 0 else -1
        if self.particlesPerEvent() == 3:
            dpdg = self.decayPDG()
            d1, d2 = (22, 22) if dpdg == 22 else (s1 * dpdg, -s1 * dpdg)
            parent = tuple(a[i] + b[i] for i in range(4))
            return [(pdg, 23, 0, parent), (d1, 33, 1, a), (d2, 33, 1, b)]
        if not charged:
            return [(pdg, 23, 0, a), (pdg, 23, 0, b)]
        return [(s1 * pdg, 23, 0, a), (-s1 * pdg, 23, 0, b)]

    def getParticles(self):
        """The particles of the last generateEvent (UpcGenerator::getParticles)."""
        rec = getattr(self, "_last_record", None)
        return [] if rec is None else self.particlesOf(rec)

    def timings(self):
        v = (C.c_double * 8)()
        _check(self._L.upcg_last_timings(self._h, v, 8))
        return {"tables_ms": v[0], "lumi_ms": v[1], "xsec_ms": v[2], "nodes_ms": v[3],
                "qags_ms": v[4], "contract_ms": v[5], "project_ms": v[6], "fluxtab_ms": v[7]}

    def qagsStats(self):
        f, m, e = C.c_uint64(), C.c_uint64(), C.c_uint64()
        _check(self._L.upcg_qags_stats(self._h, C.byref(f), C.byref(m), C.byref(e)))
        return {"failures": f.value, "max_intervals": m.value, "evals": e.value}
