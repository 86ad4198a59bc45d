"""ctypes binding of libkb2pi (include/kb2pi.h).

This is the same boundary a Julia `ccall` binds (see the Julia glue in
qftdynamicsm.jl_gb300/julia/). Loading fails loudly when the shared library
has not been built: there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

import numpy as np

# KB2PI_LIB selects another build of the library (e.g. libkb2pi_debug.so, the
# build with device-side bounds checks) for the whole process
LIB_PATH = os.environ.get("KB2PI_LIB") or os.path.join(os.path.dirname(os.path.abspath(__file__)), "libkb2pi.so")

KB_OK = 0
KB_ERR = {
    -1: "KB_ERR_PARAM", -2: "KB_ERR_OOM", -3: "KB_ERR_CUDA", -4: "KB_ERR_NAN",
    -5: "KB_ERR_TIMEOUT", -6: "KB_ERR_RANGE", -7: "KB_ERR_NODEV",
}
KB_PEXP_LO, KB_PEXP_NLO_QUANTUM, KB_PEXP_NLO_CLASSICAL, KB_PEXP_NINV_LO, KB_PEXP_NINV_NLO = 0, 1, 2, 3, 4
KB_PREC_FP64, KB_PREC_MIXED = 0, 1

# every symbol include/kb2pi.h declares
EXPORTS = [
    "kb_create", "kb_create_batch", "kb_destroy", "kb_last_error", "kb_num_orbits", "kb_get_orbits",
    "kb_site_orbits", "kb_init", "kb_init_rows", "kb_step", "kb_steps", "kb_expand", "kb_measure",
    "kb_measure_enqueue", "kb_measure_take",
    "kb_get_traces", "kb_get", "kb_set", "kb_self_energies", "kb_get_sigma", "kb_window",
    "kb_checkpoint_size", "kb_checkpoint_save", "kb_checkpoint_restore", "kb_sync",
    "kb_get_stream", "kb_profile", "kb_profile_read", "kb_steps_recorded", "kb_get_tuning", "kb_set_tuning", "kb_autotune",
    "kb_adjoint", "kb_sunset_rows_noalloc",
]


class KbParams(C.Structure):
    _fields_ = [
        ("Ns", C.c_int32), ("sdim", C.c_int32), ("M", C.c_int32), ("N", C.c_int32),
        ("pexp", C.c_int32), ("precision", C.c_int32), ("device", C.c_int32), ("flags", C.c_int32),
        ("dt", C.c_double), ("lam", C.c_double), ("mass2", C.c_double), ("mass", C.c_double),
    ]


class KbMeasScalars(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("time", "E", "E_pot", "E_kin", "E_mem", "M2")]

    def as_dict(self):
        return {n: getattr(self, n) for n, _ in self._fields_}


class KbTuning(C.Structure):
    _fields_ = [("memint_variant", C.c_int32), ("sunset_grid", C.c_int32), ("batch_order", C.c_int32),
                ("sunset_variant", C.c_int32), ("memint_split", C.c_int32), ("memint_bulk", C.c_int32),
                ("test_no_tiles", C.c_int32), ("memint_compensated", C.c_int32), ("batch_overlap", C.c_int32),
                ("memint_persistent", C.c_int32)]

    def as_dict(self):
        return {"memint_variant": self.memint_variant, "sunset_grid": self.sunset_grid,
                "batch_order": self.batch_order, "sunset_variant": self.sunset_variant,
                "memint_split": self.memint_split, "memint_bulk": self.memint_bulk,
                "test_no_tiles": self.test_no_tiles, "memint_compensated": self.memint_compensated,
                "batch_overlap": self.batch_overlap, "memint_persistent": self.memint_persistent}


class KbError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{KB_ERR.get(code, code)}: {msg}")
        self.code = code


_LIB = None
_LOCK = threading.Lock()


def load_library(path: str | None = None):
    """Load libkb2pi.so (raises if it was not built)."""
    global _LIB
    with _LOCK:
        if _LIB is not None:
            return _LIB
        p = path or LIB_PATH
        if not os.path.exists(p):
            raise ImportError(f"{p} is missing: build the CUDA library first (python -c 'import __graft_entry__ as g; g.build()')")
        lib = C.CDLL(p)
        P = C.POINTER
        d, i32, i64, vp = C.c_double, C.c_int32, C.c_int64, C.c_void_p
        dp = P(d)
        sig = {
            "kb_create": (C.c_int, [P(KbParams), P(vp)]),
            "kb_create_batch": (C.c_int, [P(KbParams), i32, P(vp)]),
            "kb_destroy": (None, [vp]),
            "kb_last_error": (C.c_char_p, [vp]),
            "kb_num_orbits": (C.c_int, [vp, i32, P(i32)]),
            "kb_get_orbits": (C.c_int, [vp, i32, P(i32), dp, P(i64)]),
            "kb_site_orbits": (C.c_int, [vp, i32, P(i32)]),
            "kb_init": (C.c_int, [vp, i32, dp, d]),
            "kb_init_rows": (C.c_int, [vp, i32, dp, dp, dp]),
            "kb_step": (C.c_int, [vp, i32]),
            "kb_steps": (C.c_int, [vp, i32, i32, i32, P(KbMeasScalars), i32]),
            "kb_expand": (C.c_int, [vp]),
            "kb_measure": (C.c_int, [vp, i32, i32, P(KbMeasScalars), dp, dp, dp, dp, dp]),
            "kb_measure_enqueue": (C.c_int, [vp, i32, i32]),
            "kb_measure_take": (C.c_int, [vp, i32, i32, P(KbMeasScalars), dp, dp, dp, dp, dp]),
            "kb_get_traces": (C.c_int, [vp, i32, dp, dp, dp, dp]),
            "kb_get": (C.c_int, [vp, i32, i32, i32, i32, dp]),
            "kb_set": (C.c_int, [vp, i32, i32, i32, i32, dp]),
            "kb_self_energies": (C.c_int, [vp, i32]),
            "kb_get_sigma": (C.c_int, [vp, i32, i32, i32, dp]),
            "kb_window": (C.c_int, [vp, i32, P(i32), P(i32)]),
            "kb_checkpoint_size": (C.c_int, [vp, P(C.c_size_t)]),
            "kb_checkpoint_save": (C.c_int, [vp, vp, C.c_size_t]),
            "kb_checkpoint_restore": (C.c_int, [vp, vp, C.c_size_t]),
            "kb_sync": (C.c_int, [vp]),
            "kb_get_stream": (C.c_int, [vp, P(vp)]),
            "kb_profile": (C.c_int, [vp, i32]),
            "kb_profile_read": (C.c_int, [vp, dp, P(i64)]),
            "kb_steps_recorded": (C.c_int, [vp, i32, i32, i32, P(KbMeasScalars), dp, i32, P(i32)]),
            "kb_get_tuning": (C.c_int, [vp, P(KbTuning)]),
            "kb_set_tuning": (C.c_int, [vp, P(KbTuning)]),
            "kb_autotune": (C.c_int, [vp, i32, P(KbTuning), dp]),
            "kb_adjoint": (C.c_int, [vp, dp, d, i32, dp, d, i32, dp, dp, dp, dp, dp]),
            "kb_sunset_rows_noalloc": (C.c_int, [i32, i32, d, i32, i32, vp, vp, vp, vp, vp]),
        }
        for name, (res, args) in sig.items():
            f = getattr(lib, name)
            f.restype = res
            f.argtypes = args
        _LIB = lib
    return _LIB


def dptr(a):
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_double))


class Handle:
    """Owner of one kb_handle (one or several runs in lock-step)."""

    def __init__(self, params: list[KbParams]):
        self.lib = load_library()
        arr = (KbParams * len(params))(*params)
        h = C.c_void_p()
        rc = self.lib.kb_create_batch(arr, len(params), C.byref(h))
        if rc != KB_OK:
            raise KbError(rc, self.lib.kb_last_error(None).decode())
        self.h = h
        self.nruns = len(params)
        self.S = []
        for r in range(self.nruns):
            s = C.c_int32()
            self._check(self.lib.kb_num_orbits(self.h, r, C.byref(s)))
            self.S.append(s.value)

    def _check(self, rc):
        if rc != KB_OK:
            raise KbError(rc, self.lib.kb_last_error(self.h).decode())

    def close(self):
        if getattr(self, "h", None):
            self.lib.kb_destroy(self.h)
            self.h = None

    def __del__(self):  # pragma: no cover
        try:
            self.close()
        except Exception:
            pass

    def orbits(self, run=0):
        S = self.S[run]
        rep = np.zeros((S, 3), np.int32)
        k2 = np.zeros(S)
        deg = np.zeros(S, np.int64)
        self._check(self.lib.kb_get_orbits(self.h, run, rep.ctypes.data_as(C.POINTER(C.c_int32)), dptr(k2),
                                           deg.ctypes.data_as(C.POINTER(C.c_int64))))
        return rep, k2, deg

    def site_orbits(self, run, V):
        out = np.zeros(V, np.int32)
        self._check(self.lib.kb_site_orbits(self.h, run, out.ctypes.data_as(C.POINTER(C.c_int32))))
        return out

    def init(self, run, n, init_mass):
        n = np.ascontiguousarray(n, np.float64)
        self._check(self.lib.kb_init(self.h, run, dptr(n), float(init_mass)))

    def init_rows(self, run, F11, F21, F22):
        a = [np.ascontiguousarray(x, np.float64) for x in (F11, F21, F22)]
        self._check(self.lib.kb_init_rows(self.h, run, *[dptr(x) for x in a]))

    def step(self, t):
        self._check(self.lib.kb_step(self.h, int(t)))

    def steps(self, t0, count, measure_every=0):
        nm = (count + measure_every - 1) // measure_every if measure_every > 0 else 0
        cap = max(1, nm * self.nruns)
        out = (KbMeasScalars * cap)()
        self._check(self.lib.kb_steps(self.h, int(t0), int(count), int(measure_every), out, cap))
        return [[out[r * nm + i].as_dict() for i in range(nm)] for r in range(self.nruns)]

    def steps_recorded(self, t0, count, measure_every, arrays=True):
        """kb_steps_recorded: evolve count steps from t0 with the measurements of every
        measure_every-th step recorded on the device; returns per measured step a list
        (one dict per run) of the scalars and, with arrays=True, F, ddF, n, omega, c."""
        rem = (t0 - 2) % measure_every
        tf = t0 + (0 if rem == 0 else measure_every - rem)
        nmeas = max(0, (t0 + count - 1 - tf) // measure_every + 1) if tf <= t0 + count - 1 else 0
        cap = max(1, nmeas)
        out = (KbMeasScalars * (cap * self.nruns))()
        per = [5 * S for S in self.S]
        arr = np.zeros(cap * sum(per)) if arrays else None
        nrec = C.c_int32()
        self._check(self.lib.kb_steps_recorded(self.h, int(t0), int(count), int(measure_every), out, dptr(arr),
                                               int(cap), C.byref(nrec)))
        res = []
        off = 0
        for m in range(nrec.value):
            row = []
            for r in range(self.nruns):
                d = out[m * self.nruns + r].as_dict()
                d["t"] = tf + m * measure_every
                if arrays:
                    a = arr[off:off + per[r]].reshape(5, self.S[r])
                    for q, k in enumerate(("F", "ddF", "n", "omega", "c")):
                        d[k] = a[q].copy()
                off += per[r]
                row.append(d)
            res.append(row)
        return res

    def expand(self):
        self._check(self.lib.kb_expand(self.h))

    def measure(self, run, t, arrays=True):
        S = self.S[run]
        s = KbMeasScalars()
        arrs = {k: np.zeros(S) for k in ("F", "ddF", "n", "omega", "c")} if arrays else {}
        self._check(self.lib.kb_measure(self.h, run, int(t), C.byref(s), *[dptr(arrs.get(k)) for k in
                                                                            ("F", "ddF", "n", "omega", "c")]))
        out = s.as_dict()
        out.update(arrs)
        return out

    def measure_enqueue(self, run, t):
        """Queue step t's measurement (t = the last evolved step) without waiting."""
        self._check(self.lib.kb_measure_enqueue(self.h, run, int(t)))

    def measure_take(self, run, t, arrays=True):
        """The measurement queued by measure_enqueue(run, t): same dict as measure()."""
        S = self.S[run]
        s = KbMeasScalars()
        arrs = {k: np.zeros(S) for k in ("F", "ddF", "n", "omega", "c")} if arrays else {}
        self._check(self.lib.kb_measure_take(self.h, run, int(t), C.byref(s),
                                             *[dptr(arrs.get(k)) for k in ("F", "ddF", "n", "omega", "c")]))
        out = s.as_dict()
        out.update(arrs)
        return out

    def window(self, run=0):
        a, b = C.c_int32(), C.c_int32()
        self._check(self.lib.kb_window(self.h, run, C.byref(a), C.byref(b)))
        return a.value, b.value

    def traces(self, run=0):
        tmin, tmax = self.window(run)
        n = tmax - tmin
        out = {k: np.zeros(n) for k in ("Fonet", "ronet", "SigF", "Sigr")}
        self._check(self.lib.kb_get_traces(self.h, run, dptr(out["Fonet"]), dptr(out["ronet"]),
                                           dptr(out["SigF"]), dptr(out["Sigr"])))
        return out

    def get(self, run, which, a, b):
        out = np.zeros(self.S[run])
        self._check(self.lib.kb_get(self.h, run, which, int(a), int(b), dptr(out)))
        return out

    def set(self, run, which, a, b, vals):
        v = np.ascontiguousarray(vals, np.float64)
        self._check(self.lib.kb_set(self.h, run, which, int(a), int(b), dptr(v)))

    def self_energies(self, tmone):
        self._check(self.lib.kb_self_energies(self.h, int(tmone)))

    def sigma(self, run, which, z):
        out = np.zeros(self.S[run])
        self._check(self.lib.kb_get_sigma(self.h, run, which, int(z), dptr(out)))
        return out

    def checkpoint(self):
        n = C.c_size_t()
        self._check(self.lib.kb_checkpoint_size(self.h, C.byref(n)))
        buf = np.empty(n.value, np.uint8)
        self._check(self.lib.kb_checkpoint_save(self.h, buf.ctypes.data_as(C.c_void_p), n.value))
        return buf

    def restore(self, buf):
        self._check(self.lib.kb_checkpoint_restore(self.h, buf.ctypes.data_as(C.c_void_p), buf.nbytes))

    def sync(self):
        self._check(self.lib.kb_sync(self.h))

    def stream(self):
        s = C.c_void_p()
        self._check(self.lib.kb_get_stream(self.h, C.byref(s)))
        return s.value

    def profile(self, enable=True):
        self._check(self.lib.kb_profile(self.h, 1 if enable else 0))

    def profile_read(self):
        ms = np.zeros(2)
        n = np.zeros(2, np.int64)
        self._check(self.lib.kb_profile_read(self.h, dptr(ms), n.ctypes.data_as(C.POINTER(C.c_int64))))
        return {"sunset": (ms[0], int(n[0])), "memint": (ms[1], int(n[1]))}

    def tuning(self):
        out = KbTuning()
        self._check(self.lib.kb_get_tuning(self.h, C.byref(out)))
        return out.as_dict()

    def set_tuning(self, memint_variant=None, sunset_grid=None, batch_order=None, sunset_variant=None,
                   memint_split=None, memint_bulk=None, test_no_tiles=None, memint_compensated=None,
                   batch_overlap=None, memint_persistent=None):
        cur = KbTuning()
        self._check(self.lib.kb_get_tuning(self.h, C.byref(cur)))
        if memint_variant is not None:
            cur.memint_variant = int(memint_variant)
        if sunset_grid is not None:
            cur.sunset_grid = int(sunset_grid)
        if batch_order is not None:
            cur.batch_order = int(batch_order)
        if sunset_variant is not None:
            cur.sunset_variant = int(sunset_variant)
        if memint_split is not None:
            cur.memint_split = int(memint_split)
        if memint_bulk is not None:
            cur.memint_bulk = int(memint_bulk)
        if test_no_tiles is not None:
            cur.test_no_tiles = int(test_no_tiles)
        if memint_compensated is not None:
            cur.memint_compensated = int(memint_compensated)
        if batch_overlap is not None:
            cur.batch_overlap = int(batch_overlap)
        if memint_persistent is not None:
            cur.memint_persistent = int(memint_persistent)
        self._check(self.lib.kb_set_tuning(self.h, C.byref(cur)))

    def autotune(self, trials=3):
        """Time the candidate launch configurations on the last evolved step; keep the fastest."""
        out = KbTuning()
        ms = C.c_double()
        self._check(self.lib.kb_autotune(self.h, int(trials), C.byref(out), C.byref(ms)))
        d = out.as_dict()
        d["ms_per_step"] = ms.value
        return d

    def adjoint(self, n_init, init_mass, t_final, w_n=None, w_E=0.0, ckpt_every=20):
        """Gradients of sum_k w_n[k] n(k, t_final) + w_E E(t_final) (kb_adjoint).

        Returns {"loss", "lambda", "mass2", "n_init" (per orbit), "init_mass"}.
        The handle's state is consumed (call init() before stepping again)."""
        n0 = np.ascontiguousarray(n_init, dtype=np.float64)
        wn = None if w_n is None else np.ascontiguousarray(w_n, dtype=np.float64)
        gl, gm, gi, L = C.c_double(), C.c_double(), C.c_double(), C.c_double()
        gn = np.zeros(n0.shape[0])
        self._check(self.lib.kb_adjoint(self.h, dptr(n0), float(init_mass), int(t_final), dptr(wn), float(w_E),
                                        int(ckpt_every), C.byref(gl), C.byref(gm), dptr(gn), C.byref(gi),
                                        C.byref(L)))
        return {"loss": L.value, "lambda": gl.value, "mass2": gm.value, "n_init": gn, "init_mass": gi.value}
