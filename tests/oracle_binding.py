"""ctypes binding to the oracle (oracle/_build/libwqlref.so) for the tests."""
import ctypes
import os

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
_LIB = None

STREAMS = ["Uface", "Vface", "S", "Uhat", "Vhat", "Svel", "trup", "state"]
NCOMP = {"Uface": 9, "Vface": 9, "S": 4, "Uhat": 6, "Vhat": 6, "Svel": 3, "trup": 1, "state": 1}


def lib():
    global _LIB
    if _LIB is None:
        L = ctypes.CDLL(os.path.join(ROOT, "oracle", "_build", "libwqlref.so"))
        L.wqlref_create.restype = ctypes.c_void_p
        L.wqlref_create.argtypes = [ctypes.c_char_p]
        L.wqlref_last_error.restype = ctypes.c_char_p
        vp = ctypes.c_void_p
        L.wqlref_destroy.argtypes = [vp]
        L.wqlref_step.argtypes = [vp, ctypes.c_int]
        L.wqlref_frame_count.argtypes = [vp]
        L.wqlref_get_frames.argtypes = [vp, ctypes.c_int, vp]
        L.wqlref_get_field.argtypes = [vp, ctypes.c_int, ctypes.c_int, vp]
        L.wqlref_set_field.argtypes = [vp, ctypes.c_int, ctypes.c_int, vp]
        L.wqlref_get_geom.argtypes = [vp, ctypes.c_int, ctypes.c_int, vp]
        L.wqlref_get_iface.argtypes = [vp, ctypes.c_int, ctypes.c_int, vp]
        L.wqlref_get_face.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, vp]
        L.wqlref_mms_norms.argtypes = [vp, ctypes.c_int, vp, vp]
        L.wqlref_info.argtypes = [vp, vp, vp, vp, vp, vp]
        L.wqlref_create_ex.restype = ctypes.c_void_p
        L.wqlref_create_ex.argtypes = [ctypes.c_char_p] + [vp] * 9
        L.wqlref_station_count.argtypes = [vp, ctypes.c_int, ctypes.POINTER(ctypes.c_int)]
        L.wqlref_station_index.argtypes = [vp, ctypes.c_int, vp]
        L.wqlref_get_seismograms.argtypes = [vp, ctypes.c_int, vp]
        L.wqlref_fd_matrix.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, vp]
        L.wqlref_up_table.argtypes = [ctypes.c_int, ctypes.c_char_p, vp, vp, vp]
        L.wqlref_up_matrix.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, vp]
        _LIB = L
    return _LIB


class Oracle:
    """One reference-semantics domain (two blocks, one fault) on the CPU."""

    def __init__(self, in_path=None, text=None, media=None):
        L = lib()
        if text is None:
            h = L.wqlref_create(str(in_path).encode())
        else:
            m = media or {}
            self._keep = []

            def ptr(a):
                if a is None:
                    return None
                a = np.ascontiguousarray(a, dtype=np.float64).ravel()
                self._keep.append(a)
                return a.ctypes.data

            pair = lambda k: m.get(k) or (None, None)  # noqa: E731
            h = L.wqlref_create_ex(text.encode(), ptr(m.get("fault_offset")), ptr(pair("topo_offset")[0]),
                                   ptr(pair("topo_offset")[1]), ptr(pair("lam")[0]), ptr(pair("mu")[0]),
                                   ptr(pair("rho")[0]), ptr(pair("lam")[1]), ptr(pair("mu")[1]),
                                   ptr(pair("rho")[1]))
        if not h:
            raise RuntimeError(L.wqlref_last_error().decode())
        self.h = ctypes.c_void_p(h)
        dims = (ctypes.c_int * 6)()
        dt, t = ctypes.c_double(), ctypes.c_double()
        nt, ns = ctypes.c_int(), ctypes.c_int()
        L.wqlref_info(self.h, dims, ctypes.byref(dt), ctypes.byref(t), ctypes.byref(nt), ctypes.byref(ns))
        self.dims = [tuple(dims[3 * b:3 * b + 3]) for b in range(2)]
        self.dt = dt.value
        self.nt = nt.value

    def __del__(self):
        if getattr(self, "h", None) is not None and _LIB is not None:
            _LIB.wqlref_destroy(self.h)
            self.h = None

    def step(self, n=1):
        lib().wqlref_step(self.h, n)

    def field(self, block, comp):
        nq, nr, ns = self.dims[block]
        out = np.empty(nq * nr * ns, np.float64)
        lib().wqlref_get_field(self.h, block, comp, out.ctypes.data)
        return out.reshape(ns, nr, nq)

    def fields(self, block):
        return np.stack([self.field(block, c) for c in range(9)])

    def set_field(self, block, comp, arr):
        a = np.ascontiguousarray(arr, dtype=np.float64)
        lib().wqlref_set_field(self.h, block, comp, a.ctypes.data)

    def geom(self, block, what):
        nq, nr, ns = self.dims[block]
        out = np.empty(nq * nr * ns, np.float64)
        lib().wqlref_get_geom(self.h, block, what, out.ctypes.data)
        return out.reshape(ns, nr, nq)

    def face_vectors(self, block, side):
        """(n, m, l) unit vectors of face `side` (1..6) of `block`, each (3, nb, na)."""
        nq, nr, ns = self.dims[block]
        na, nb = {1: (nr, ns), 2: (nq, ns), 3: (nq, nr)}[(side + 1) // 2]
        out = np.empty((9, nb, na), np.float64)
        for w in range(9):
            assert lib().wqlref_get_face(self.h, block, side, w, out[w].ctypes.data) == 0
        return out[0:3], out[3:6], out[6:9]

    def mms_norms(self, block):
        """Per component: sum of (F - u_exact)^2 and of u_exact^2 over the block."""
        e, r = np.empty(9), np.empty(9)
        assert lib().wqlref_mms_norms(self.h, block, e.ctypes.data, r.ctypes.data) == 0
        return e, r

    def iface(self, block, what):
        nr, ns = self.dims[0][1], self.dims[0][2]
        out = np.empty(nr * ns, np.float64)
        lib().wqlref_get_iface(self.h, block, what, out.ctypes.data)
        return out.reshape(ns, nr)

    def stations(self, block):
        """(1-based grid indices (n, 3), seismograms (records, n, 4) of t, vx, vy, vz)."""
        nrec = ctypes.c_int()
        n = lib().wqlref_station_count(self.h, block, ctypes.byref(nrec))
        ijk = np.empty(3 * n, np.int32)
        lib().wqlref_station_index(self.h, block, ijk.ctypes.data)
        rec = np.empty(nrec.value * n * 4, np.float64)
        lib().wqlref_get_seismograms(self.h, block, rec.ctypes.data)
        return ijk.reshape(n, 3), rec.reshape(nrec.value, n, 4)

    def frames(self, name):
        nf = lib().wqlref_frame_count(self.h)
        nr, ns = self.dims[0][1], self.dims[0][2]
        out = np.empty(nf * NCOMP[name] * nr * ns, np.float32)
        lib().wqlref_get_frames(self.h, STREAMS.index(name), out.ctypes.data)
        return out.reshape(nf, NCOMP[name], ns, nr)


def up_tables():
    """[(fd_type, order, closure rows, tau0)] of the oracle's table operators."""
    out = []
    k = 0
    while True:
        fd = ctypes.create_string_buffer(16)
        o, R, t = ctypes.c_int(), ctypes.c_int(), ctypes.c_double()
        if lib().wqlref_up_table(k, fd, ctypes.byref(o), ctypes.byref(R), ctypes.byref(t)) < 0:
            return out
        out.append((fd.value.decode(), o.value, R.value, t.value))
        k += 1


def up_matrix(k, plus, n, axis=0, interior=False):
    """Dense n x n D+ (plus) or D- (times h) of table operator k along an axis;
    interior: the interior routine's rows inside instead of the near-boundary
    routine's."""
    D = np.zeros((n, n))
    assert lib().wqlref_up_matrix(k, int(plus), axis, int(interior), n, D.ctypes.data) == 0
    return D


def fd_matrix(fd, plus, n):
    """Dense n x n first-derivative operator of the oracle (times h): fd 0
    the traditional SBP-6 D, fd 1 the upwind D+ (plus) or D- of order 6."""
    D = np.zeros((n, n))
    assert lib().wqlref_fd_matrix(fd, int(plus), n, D.ctypes.data) == 0
    return D
