"""Python binding of the C ABI in include/wql.h (ctypes).

Mirrors the reference's driver loop (src/main.f90:63-129): build a domain
from a `.in` file, advance it step by step, read fields and the fault output
streams.  The library must have been built (wql_build.build()); there is no
fallback path -- without the CUDA library every call raises.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libwql.so")

FP64 = 0
FP32C = 1
STREAMS = ["Uface", "Vface", "S", "Uhat", "Vhat", "Svel", "trup", "state"]
NCOMP = {"Uface": 9, "Vface": 9, "S": 4, "Uhat": 6, "Vhat": 6, "Svel": 3, "trup": 1, "state": 1}
ERRORS = {1: "WQL_E_INPUT", 2: "WQL_E_OOM", 3: "WQL_E_CUDA", 4: "WQL_E_NAN", 5: "WQL_E_SOLVER",
          6: "WQL_E_STATE"}
EXPORTS = ["wql_last_error", "wql_ctx_create", "wql_ctx_destroy", "wql_scenario_create_from_in",
           "wql_scenario_create_from_text", "wql_scenario_create_ex", "wql_scenario_destroy", "wql_step", "wql_sync",
           "wql_get_info", "wql_get_field", "wql_set_field", "wql_get_iface", "wql_frame_count",
           "wql_get_frames", "wql_scenario_stream", "wql_launches_per_step", "wql_profile",
           "wql_kernel_times", "wql_set_tuning", "wql_get_field_noalloc", "wql_station_count",
           "wql_station_index", "wql_get_seismograms", "wql_batch_create", "wql_batch_destroy",
           "wql_batch_add", "wql_batch_remove", "wql_batch_step", "wql_batch_stream",
           "wql_estimate_device_bytes", "wql_server_create", "wql_server_submit", "wql_server_wait",
           "wql_server_result", "wql_server_release", "wql_server_stats", "wql_server_destroy",
           "wql_autotune", "wql_write_outputs", "wql_write_block_grids", "wql_stage", "wql_mms_norms"]


class Media(ctypes.Structure):
    _fields_ = [("fault_offset", ctypes.c_void_p), ("topo_offset", ctypes.c_void_p * 2),
                ("lam", ctypes.c_void_p * 2), ("mu", ctypes.c_void_p * 2), ("rho", ctypes.c_void_p * 2)]


class WqlError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


class Info(ctypes.Structure):
    _fields_ = [("nq", ctypes.c_int * 2), ("nr", ctypes.c_int * 2), ("ns", ctypes.c_int * 2),
                ("dt", ctypes.c_double), ("t", ctypes.c_double), ("nt", ctypes.c_int),
                ("nstep", ctypes.c_int), ("precision", ctypes.c_int), ("frames", ctypes.c_int),
                ("device_bytes", ctypes.c_longlong)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise WqlError(3, f"{LIB_PATH} is missing; build it with wql_build.build()")
        L = ctypes.CDLL(LIB_PATH)
        vp, ci = ctypes.c_void_p, ctypes.c_int
        L.wql_last_error.argtypes = [ctypes.c_char_p, ctypes.c_size_t]
        L.wql_ctx_create.argtypes = [ci, ctypes.POINTER(vp)]
        L.wql_ctx_destroy.argtypes = [vp]
        L.wql_scenario_create_from_in.argtypes = [vp, ctypes.c_char_p, ci, ctypes.POINTER(vp)]
        L.wql_scenario_create_from_text.argtypes = [vp, ctypes.c_char_p, ctypes.c_char_p, ci, ctypes.POINTER(vp)]
        L.wql_scenario_create_ex.argtypes = [vp, ctypes.c_char_p, ctypes.c_char_p, ci, ctypes.POINTER(Media),
                                             ctypes.POINTER(vp)]
        L.wql_scenario_destroy.argtypes = [vp]
        L.wql_step.argtypes = [vp, ci]
        L.wql_sync.argtypes = [vp, ci]
        L.wql_get_info.argtypes = [vp, ctypes.POINTER(Info)]
        L.wql_get_field.argtypes = [vp, ci, ci, vp]
        L.wql_set_field.argtypes = [vp, ci, ci, vp]
        L.wql_get_field_noalloc.argtypes = [vp, ci, ci, vp]
        L.wql_station_count.argtypes = [vp, ci, ctypes.POINTER(ci), ctypes.POINTER(ci)]
        L.wql_batch_create.argtypes = [vp, ctypes.POINTER(vp)]
        ll = ctypes.c_longlong
        L.wql_estimate_device_bytes.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ci, ctypes.POINTER(ll),
                                                ctypes.POINTER(ll)]
        L.wql_server_create.argtypes = [vp, ll, ci, ctypes.POINTER(vp)]
        L.wql_server_submit.argtypes = [vp, ctypes.c_char_p, ci, vp, ci, ctypes.POINTER(ll)]
        L.wql_server_wait.argtypes = [vp, ll, ctypes.c_double, ctypes.POINTER(ci)]
        L.wql_server_result.argtypes = [vp, ll, ci, ctypes.POINTER(ci), ctypes.POINTER(ci), vp, vp]
        L.wql_server_release.argtypes = [vp, ll]
        L.wql_server_stats.argtypes = [vp, ctypes.POINTER(ll), ctypes.POINTER(ll), ctypes.POINTER(ll),
                                       ctypes.POINTER(ll)]
        L.wql_server_destroy.argtypes = [vp]
        L.wql_autotune.argtypes = [vp, ci, ctypes.POINTER(ci), ctypes.POINTER(ci)]
        L.wql_batch_destroy.argtypes = [vp]
        L.wql_batch_add.argtypes = [vp, vp]
        L.wql_batch_remove.argtypes = [vp, vp]
        L.wql_batch_step.argtypes = [vp, ci]
        L.wql_batch_stream.argtypes = [vp, ctypes.POINTER(ctypes.c_size_t)]
        L.wql_station_index.argtypes = [vp, ci, vp]
        L.wql_get_seismograms.argtypes = [vp, ci, vp]
        L.wql_write_outputs.argtypes = [vp, ctypes.c_char_p]
        L.wql_stage.argtypes = [vp, ci]
        L.wql_write_block_grids.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p]
        L.wql_get_iface.argtypes = [vp, ci, ci, vp]
        L.wql_mms_norms.argtypes = [vp, ci, vp, vp]
        L.wql_frame_count.argtypes = [vp, ctypes.POINTER(ci)]
        L.wql_get_frames.argtypes = [vp, ci, vp]
        L.wql_scenario_stream.argtypes = [vp, ctypes.POINTER(ctypes.c_size_t)]
        L.wql_launches_per_step.argtypes = [vp, ctypes.POINTER(ci)]
        L.wql_profile.argtypes = [vp, ci]
        L.wql_set_tuning.argtypes = [vp, ci, ci]
        cd = ctypes.POINTER(ctypes.c_double)
        L.wql_kernel_times.argtypes = [vp, ci, cd, ctypes.POINTER(ci)]
        _lib = L
    return _lib


def _check(rc):
    if rc != 0:
        buf = ctypes.create_string_buffer(1024)
        lib().wql_last_error(buf, 1024)
        raise WqlError(rc, buf.value.decode())


def _media_struct(media):
    """A Media struct over contiguous FP64 copies of the arrays (returned
    alongside so they stay alive for the call)."""
    keep = []

    def ptr(a):
        if a is None:
            return None
        a = np.ascontiguousarray(a, dtype=np.float64).ravel()
        keep.append(a)
        return a.ctypes.data

    m = Media()
    m.fault_offset = ptr(media.get("fault_offset"))
    for key in ("topo_offset", "lam", "mu", "rho"):
        pair = media.get(key) or (None, None)
        arr = getattr(m, key)
        for b in range(2):
            arr[b] = ptr(pair[b])
    return m, keep


class Context:
    def __init__(self, device=0):
        self.h = ctypes.c_void_p()
        _check(lib().wql_ctx_create(device, ctypes.byref(self.h)))

    def close(self):
        if self.h:
            lib().wql_ctx_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Scenario:
    """One two-block domain on the GPU (the reference's `domain_type`)."""

    def __init__(self, ctx, in_path=None, text=None, precision=FP64, base_dir=None, media=None):
        """media: optional dict with 'fault_offset' (nr*ns), 'topo_offset'
        (pair of nq*ns), 'lam'/'mu'/'rho' (pairs of per-point arrays)."""
        self.ctx = ctx
        self.h = ctypes.c_void_p()
        if media is not None:
            if text is None:
                with open(in_path) as f:
                    text = f.read()
            m, keep = _media_struct(media)
            _check(lib().wql_scenario_create_ex(ctx.h, text.encode(),
                                                base_dir.encode() if base_dir else None, precision,
                                                ctypes.byref(m), ctypes.byref(self.h)))
        elif text is not None:
            _check(lib().wql_scenario_create_from_text(
                ctx.h, text.encode(), base_dir.encode() if base_dir else None, precision,
                ctypes.byref(self.h)))
        else:
            _check(lib().wql_scenario_create_from_in(ctx.h, str(in_path).encode(), precision,
                                                     ctypes.byref(self.h)))
        self.precision = precision

    def close(self):
        if self.h:
            lib().wql_scenario_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def info(self):
        i = Info()
        _check(lib().wql_get_info(self.h, ctypes.byref(i)))
        return i

    @property
    def dims(self):
        i = self.info()
        return [(i.nq[b], i.nr[b], i.ns[b]) for b in range(2)]

    def step(self, n=1):
        _check(lib().wql_step(self.h, n))

    def sync(self, check_nan=False):
        _check(lib().wql_sync(self.h, 1 if check_nan else 0))

    def field(self, block, comp):
        nq, nr, ns = self.dims[block]
        out = np.empty(nq * nr * ns, np.float64)
        _check(lib().wql_get_field(self.h, block, comp, out.ctypes.data))
        return out.reshape(ns, nr, nq)

    def stations(self, block):
        """(1-based grid indices (n, 3), records (nrec, n, 4) of t, vx, vy, vz)."""
        n, nrec = ctypes.c_int(), ctypes.c_int()
        _check(lib().wql_station_count(self.h, block, ctypes.byref(n), ctypes.byref(nrec)))
        ijk = np.empty(3 * n.value, np.int32)
        _check(lib().wql_station_index(self.h, block, ijk.ctypes.data))
        rec = np.empty(nrec.value * n.value * 4, np.float64)
        _check(lib().wql_get_seismograms(self.h, block, rec.ctypes.data))
        return ijk.reshape(n.value, 3), rec.reshape(nrec.value, n.value, 4)

    def stage(self, stage):
        """One RK stage (1..5, in order) of the current step (wql_stage)."""
        _check(lib().wql_stage(self.h, stage))

    def write_outputs(self, out_dir):
        """The fault streams and station files so far, in the reference's
        file formats, under out_dir (wql_write_outputs)."""
        _check(lib().wql_write_outputs(self.h, os.fsencode(str(out_dir))))

    def field_noalloc(self, block, comp):
        """As field(), through wql_get_field_noalloc (no device allocation)."""
        nq, nr, ns = self.dims[block]
        out = np.empty(nq * nr * ns, np.float64)
        _check(lib().wql_get_field_noalloc(self.h, block, comp, out.ctypes.data))
        return out.reshape(ns, nr, nq)

    def fields(self, block):
        return np.stack([self.field(block, c) for c in range(9)])

    def set_field(self, block, comp, arr):
        a = np.ascontiguousarray(arr, dtype=np.float64)
        _check(lib().wql_set_field(self.h, block, comp, a.ctypes.data))

    def iface(self, copy, what):
        nr, ns = self.dims[0][1], self.dims[0][2]
        out = np.empty(nr * ns, np.float64)
        _check(lib().wql_get_iface(self.h, copy, what, out.ctypes.data))
        return out.reshape(ns, nr)

    def mms_norms(self, block):
        """Per component: sum of (F - u_exact)^2 and of u_exact^2 over the block."""
        e, r = np.empty(9), np.empty(9)
        _check(lib().wql_mms_norms(self.h, block, e.ctypes.data, r.ctypes.data))
        return e, r

    def frame_count(self):
        n = ctypes.c_int()
        _check(lib().wql_frame_count(self.h, ctypes.byref(n)))
        return n.value

    def frames(self, name):
        nf = self.frame_count()
        nr, ns = self.dims[0][1], self.dims[0][2]
        out = np.empty(nf * NCOMP[name] * nr * ns, np.float32)
        _check(lib().wql_get_frames(self.h, STREAMS.index(name), out.ctypes.data))
        return out.reshape(nf, NCOMP[name], ns, nr)

    def stream(self):
        s = ctypes.c_size_t()
        _check(lib().wql_scenario_stream(self.h, ctypes.byref(s)))
        return s.value

    def launches_per_step(self):
        n = ctypes.c_int()
        _check(lib().wql_launches_per_step(self.h, ctypes.byref(n)))
        return n.value

    def profile(self, enable=True):
        _check(lib().wql_profile(self.h, 1 if enable else 0))

    def kernel_times(self):
        """{'interface' | 'stencil' | 'corrections': (ms_total, launches)} since profile(True)."""
        out = {}
        for kind, name in enumerate(("interface", "stencil", "corrections")):
            ms, n = ctypes.c_double(), ctypes.c_int()
            _check(lib().wql_kernel_times(self.h, kind, ctypes.byref(ms), ctypes.byref(n)))
            out[name] = (ms.value, n.value)
        return out

    def autotune(self, reps=3):
        """Time the stencil candidates and keep the fastest: (variant, schunk)."""
        v, c = ctypes.c_int(), ctypes.c_int()
        _check(lib().wql_autotune(self.h, reps, ctypes.byref(v), ctypes.byref(c)))
        return v.value, c.value

    def set_tuning(self, kernel=0, schunk=0):
        _check(lib().wql_set_tuning(self.h, kernel, schunk))


class Batch:
    """Scenarios advanced together (wql_batch_*): one packed stencil launch
    per stage for all members."""

    def __init__(self, ctx):
        h = ctypes.c_void_p()
        _check(lib().wql_batch_create(ctx.h, ctypes.byref(h)))
        self.h = h.value
        self.members = []

    def add(self, scn):
        _check(lib().wql_batch_add(self.h, scn.h))
        self.members.append(scn)

    def remove(self, scn):
        _check(lib().wql_batch_remove(self.h, scn.h))
        self.members.remove(scn)

    def step(self, n=1):
        _check(lib().wql_batch_step(self.h, n))

    def stream(self):
        s = ctypes.c_size_t()
        _check(lib().wql_batch_stream(self.h, ctypes.byref(s)))
        return s.value

    def close(self):
        if self.h:
            lib().wql_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def estimate_device_bytes(text, precision=FP32C):
    """(resident, peak) device bytes a scenario of this .in text would need."""
    r, p = ctypes.c_longlong(), ctypes.c_longlong()
    _check(lib().wql_estimate_device_bytes(text.encode(), None, precision, ctypes.byref(r), ctypes.byref(p)))
    return r.value, p.value


class Server:
    """Request server (wql_server_*): admission by device-memory footprint and
    continuous batching on a worker thread."""

    def __init__(self, ctx, hbm_budget_bytes, round_steps=10):
        h = ctypes.c_void_p()
        _check(lib().wql_server_create(ctx.h, int(hbm_budget_bytes), round_steps, ctypes.byref(h)))
        self.h = h.value
        self._keep = {}

    def submit(self, text, nsteps, precision=FP32C, media=None):
        mp = None
        if media:
            mobj, keep = _media_struct(media)
            mp = ctypes.byref(mobj)
        rid = ctypes.c_longlong()
        _check(lib().wql_server_submit(self.h, text.encode(), precision, mp, nsteps, ctypes.byref(rid)))
        return rid.value

    def wait(self, rid, timeout=600.0):
        st = ctypes.c_int()
        _check(lib().wql_server_wait(self.h, rid, timeout, ctypes.byref(st)))
        return st.value

    def result(self, rid, block):
        """(seismograms (records, n, 4), (t_arrive, t_admit, t_done))."""
        n, nrec = ctypes.c_int(), ctypes.c_int()
        times = np.zeros(3)
        rc = lib().wql_server_result(self.h, rid, block, ctypes.byref(n), ctypes.byref(nrec), None,
                                     times.ctypes.data)
        if rc:
            raise WqlError(rc, "request %d failed" % rid)
        seis = np.empty(nrec.value * n.value * 4)
        _check(lib().wql_server_result(self.h, rid, block, None, None, seis.ctypes.data, None))
        return seis.reshape(nrec.value, n.value, 4), tuple(times)

    def release(self, rid):
        _check(lib().wql_server_release(self.h, rid))

    def stats(self):
        v = [ctypes.c_longlong() for _ in range(4)]
        _check(lib().wql_server_stats(self.h, *[ctypes.byref(x) for x in v]))
        return dict(zip(("completed", "queued", "active", "bytes_in_use"), (x.value for x in v)))

    def close(self):
        if self.h:
            lib().wql_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def write_block_grids(text, out_dir, base_dir=None):
    """The grids of both blocks of an .in text as block_grid_<id>.X/.Y/.Z in
    out_dir (raw FP64, q fastest), the files mesh_source = 'file' reads
    (wql_write_block_grids; host only)."""
    _check(lib().wql_write_block_grids(text.encode(), str(base_dir).encode() if base_dir else None,
                                       os.fsencode(str(out_dir))))
