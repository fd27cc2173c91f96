"""ctypes binding of libbtgpu.so (the C ABI declared in include/btgpu.h).

The library is the only compute path: when it is missing or cannot be loaded
every call raises, there is no CPU fallback.
"""

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libbtgpu.so")

BT_OK = 0
BT_ERR_INVALID = 1
BT_ERR_CUDA = 2
BT_ERR_OOM = 3
BT_ERR_NOT_CONVERGED = 4
BT_ERR_BREAKDOWN = 5
BT_ERR_TIMEOUT = 6
BT_ERR_STATE = 7
PRECISION_FP64 = 0
PRECISION_MIXED = 1
MATRICES = {"M": 0, "K": 1, "T": 2, "R": 3, "Jx": 4, "Jy": 5, "Jz": 6}
_ERRNAMES = {1: "BT_ERR_INVALID", 2: "BT_ERR_CUDA", 3: "BT_ERR_OOM", 4: "BT_ERR_NOT_CONVERGED",
             5: "BT_ERR_BREAKDOWN", 6: "BT_ERR_TIMEOUT", 7: "BT_ERR_STATE"}

# every function declared in include/btgpu.h
EXPORTS = [
    "bt_version", "bt_create", "bt_destroy", "bt_last_error", "bt_set_stream",
    "bt_mesh_upload", "bt_mesh_info", "bt_set_coefficients", "bt_set_cell_diffusion",
    "bt_assemble", "bt_set_schedule", "bt_solve", "bt_get_csr", "bt_get_matrix",
    "bt_get_dofs", "bt_get_colouring", "bt_get_solution", "bt_get_iterations", "bt_set_option",
    "bt_signal_noalloc", "bt_adjoint", "bt_solve_multi", "bt_set_cell_T2", "bt_tangent",
    "bt_set_schedule_phase", "bt_set_periodic", "bt_periodic_info", "bt_adjoint_batch", "bt_adjoint_multi",
    "bt_set_kappa_mode", "bt_set_schedule_integral", "bt_set_periodic_mode", "bt_strong_periodic_info",
    "bt_adjoint_cells", "bt_adjoint_batch_cells", "bt_solve_dev",
]


class BtError(RuntimeError):
    """A libbtgpu call returned a non-zero status."""

    def __init__(self, code, msg):
        super().__init__("%s (%d): %s" % (_ERRNAMES.get(code, "BT_ERR"), code, msg))
        self.code = code


class PeriodicInfo(C.Structure):
    _fields_ = [("active", C.c_int32), ("dir", C.c_int32 * 3), ("kappa_e", C.c_double), ("hmin", C.c_double),
                ("n_facets", C.c_int64), ("n_rows", C.c_int64), ("n_entries", C.c_int64),
                ("n_unmatched", C.c_int64)]


class MeshInfo(C.Structure):
    _fields_ = [("n_vertices", C.c_int64), ("n_cells", C.c_int64), ("n_dofs", C.c_int64),
                ("nnz", C.c_int64), ("n_interface_facets", C.c_int64),
                ("n_compartments", C.c_int32), ("n_colours", C.c_int32),
                ("sell_entries", C.c_int64), ("volume", C.c_double)]


class Stats(C.Structure):
    _fields_ = [("steps", C.c_int32), ("max_iterations", C.c_int32),
                ("total_iterations", C.c_int64), ("max_rel_residual", C.c_double),
                ("gpu_ms", C.c_double), ("refinements", C.c_int32),
                ("graph_launches", C.c_int32), ("kernel_launches", C.c_int64),
                ("stepper_ms", C.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


_lib = None

_P = C.c_void_p
_D = C.POINTER(C.c_double)
_I32 = C.POINTER(C.c_int32)


def load(path=None):
    """Load libbtgpu.so (once).  Raises if it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        raise RuntimeError("libbtgpu.so not found at %s: build it with __graft_entry__.build() "
                           "(there is no CPU fallback)" % path)
    lib = C.CDLL(path)
    sig = {
        "bt_version": (C.c_int, []),
        "bt_create": (C.c_int, [C.POINTER(_P), C.c_int]),
        "bt_destroy": (C.c_int, [_P]),
        "bt_last_error": (C.c_int, [_P, C.c_char_p, C.c_size_t]),
        "bt_set_stream": (C.c_int, [_P, _P]),
        "bt_mesh_upload": (C.c_int, [_P, _D, C.c_int64, _I32, C.c_int64, _I32, C.c_int32, _I32]),
        "bt_mesh_info": (C.c_int, [_P, C.POINTER(MeshInfo)]),
        "bt_set_coefficients": (C.c_int, [_P, _D, _D, _D]),
        "bt_set_cell_diffusion": (C.c_int, [_P, _D]),
        "bt_set_kappa_mode": (C.c_int, [_P, C.c_int32]),
        "bt_set_cell_T2": (C.c_int, [_P, _D]),
        "bt_assemble": (C.c_int, [_P]),
        "bt_set_schedule": (C.c_int, [_P, _D, _D, C.c_int32, C.c_int32, C.c_double, C.c_double]),
        "bt_solve": (C.c_int, [_P, C.c_int32, _D, _D, _I32, _D, C.c_int32, C.c_double, C.c_int32,
                               _D, _D, _D, C.POINTER(Stats)]),
        "bt_get_csr": (C.c_int, [_P, _I32, _I32]),
        "bt_get_matrix": (C.c_int, [_P, C.c_int32, _D]),
        "bt_get_dofs": (C.c_int, [_P, _I32, _I32, _D]),
        "bt_get_colouring": (C.c_int, [_P, _I32]),
        "bt_get_solution": (C.c_int, [_P, C.c_int32, _D]),
        "bt_get_iterations": (C.c_int, [_P, _I32, C.c_int64]),
        "bt_set_option": (C.c_int, [_P, C.c_char_p, C.c_double]),
        "bt_signal_noalloc": (C.c_int, [_P, _P, C.c_int64, _P, _P]),
        "bt_adjoint": (C.c_int, [_P, C.c_double, _D, C.c_int32, _D, C.c_double, C.c_int32, C.c_int32,
                                 _D, _D, _D, _D, C.POINTER(Stats)]),
        "bt_adjoint_cells": (C.c_int, [_P, C.c_double, _D, C.c_int32, _D, C.c_double, C.c_int32, C.c_int32,
                                       _D, _D, _D, _D, C.POINTER(Stats)]),
        "bt_adjoint_batch_cells": (C.c_int, [_P, C.c_int32, _D, _D, _I32, _D, C.c_double, C.c_int32, C.c_int32,
                                             _D, _D, _D, _D, C.POINTER(Stats)]),
        "bt_solve_dev": (C.c_int, [_P, C.c_int32, _P, _P, _P, _P, C.c_int32, C.c_double, C.c_int32, _P, _P,
                                   C.POINTER(C.c_double), C.POINTER(Stats)]),
        "bt_tangent": (C.c_int, [_P, C.c_double, _D, C.c_int32, _D, C.c_int32, C.c_int32, C.c_int32, C.c_double,
                                 C.c_int32, _D, _D, C.POINTER(Stats)]),
        "bt_solve_multi": (C.c_int, [C.POINTER(_P), C.c_int32, _I32, _D, _D, _I32, C.c_double, C.c_int32,
                                     _D, _D, C.POINTER(Stats)]),
        "bt_set_schedule_phase": (C.c_int, [_P, _D, C.c_int32, C.c_int32]),
        "bt_set_periodic": (C.c_int, [_P, _I32]),
        "bt_set_schedule_integral": (C.c_int, [_P, _D, _D, C.c_int32, C.c_int32]),
        "bt_set_periodic_mode": (C.c_int, [_P, C.c_int32]),
        "bt_strong_periodic_info": (C.c_int, [_P, C.POINTER(C.c_int64), C.POINTER(C.c_int64),
                                              C.POINTER(C.c_int64)]),
        "bt_periodic_info": (C.c_int, [_P, C.POINTER(PeriodicInfo)]),
        "bt_adjoint_batch": (C.c_int, [_P, C.c_int32, _D, _D, _I32, C.c_double, C.c_int32, C.c_int32,
                                       _D, _D, _D, _D, C.POINTER(Stats)]),
        "bt_adjoint_multi": (C.c_int, [C.POINTER(_P), C.c_int32, _I32, _D, _D, _I32, C.c_double, C.c_int32,
                                       C.c_int32, _D, _D, _D, _D, C.POINTER(Stats)]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def _dp(a):
    return None if a is None else a.ctypes.data_as(_D)


def _ip(a):
    return None if a is None else a.ctypes.data_as(_I32)


class Context:
    """One libbtgpu context (device memory, stream, assembled matrices)."""

    def __init__(self, device=0):
        self.lib = load()
        h = _P()
        rc = self.lib.bt_create(C.byref(h), int(device))
        if rc != BT_OK:
            raise BtError(rc, "bt_create failed (no usable CUDA device?)")
        self.h = h
        self.n_vertices = 0
        self.n_regions = 0
        self.n_compartments = 0

    def close(self):
        if getattr(self, "h", None):
            self.lib.bt_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc):
        if rc != BT_OK:
            buf = C.create_string_buffer(1024)
            self.lib.bt_last_error(self.h, buf, 1024)
            raise BtError(rc, buf.value.decode(errors="replace"))

    def set_option(self, key, value):
        self._check(self.lib.bt_set_option(self.h, key.encode(), float(value)))

    def set_stream(self, stream_ptr):
        self._check(self.lib.bt_set_stream(self.h, _P(stream_ptr) if stream_ptr else None))

    def mesh_upload(self, xyz, tets, cell_region, n_regions=None, region_compartment=None):
        xyz = np.ascontiguousarray(xyz, dtype=np.float64)
        tets = np.ascontiguousarray(tets, dtype=np.int32)
        reg = np.ascontiguousarray(cell_region, dtype=np.int32)
        if n_regions is None:
            n_regions = int(reg.max()) + 1 if len(reg) else 1
        rc_arr = None if region_compartment is None else np.ascontiguousarray(region_compartment, dtype=np.int32)
        self._check(self.lib.bt_mesh_upload(self.h, _dp(xyz), len(xyz), _ip(tets), len(tets), _ip(reg),
                                            int(n_regions), _ip(rc_arr)))
        self.n_vertices = len(xyz)
        self.n_cells = len(tets)
        self.n_regions = int(n_regions)
        self.n_compartments = self.info()["n_compartments"]

    def info(self):
        mi = MeshInfo()
        self._check(self.lib.bt_mesh_info(self.h, C.byref(mi)))
        return {k: getattr(mi, k) for k, _ in mi._fields_}

    def set_coefficients(self, D_region, invT2_region=None, kappa_pair=None):
        D = np.ascontiguousarray(np.broadcast_to(np.asarray(D_region, np.float64), (self.n_regions,)))
        iT2 = None if invT2_region is None else np.ascontiguousarray(
            np.broadcast_to(np.asarray(invT2_region, np.float64), (self.n_regions,)))
        kp = None
        if kappa_pair is not None:
            kp = np.asarray(kappa_pair, np.float64)
            if kp.ndim == 0:
                kp = np.full((self.n_regions, self.n_regions), float(kp))
            kp = np.ascontiguousarray(kp.reshape(self.n_regions, self.n_regions))
        self._check(self.lib.bt_set_coefficients(self.h, _dp(D), _dp(iT2), _dp(kp)))

    def set_kappa_mode(self, mode):
        """'facet' (one permeability per interface facet, the default) or 'cr'
        (the Crouzeix-Raviart permeability field); takes effect at assemble()."""
        self._check(self.lib.bt_set_kappa_mode(self.h, {"facet": 0, "cr": 1}[mode]))

    def set_cell_diffusion(self, D_cell6):
        arr = None if D_cell6 is None else np.ascontiguousarray(D_cell6, dtype=np.float64)
        self._check(self.lib.bt_set_cell_diffusion(self.h, _dp(arr)))

    def set_cell_T2(self, invT2_cell):
        """Per-cell 1/T2 (None clears it)."""
        arr = None if invT2_cell is None else np.ascontiguousarray(invT2_cell, dtype=np.float64)
        if arr is not None and arr.shape != (self.n_cells,):
            raise ValueError("invT2_cell must have one value per cell")
        self._check(self.lib.bt_set_cell_T2(self.h, _dp(arr)))

    def assemble(self):
        self._check(self.lib.bt_assemble(self.h))

    def set_schedule(self, f_new, f_old, dt, theta=0.5):
        fn = np.ascontiguousarray(np.atleast_2d(np.asarray(f_new, np.float64)))
        fo = np.ascontiguousarray(np.atleast_2d(np.asarray(f_old, np.float64)))
        if fn.shape != fo.shape:
            raise ValueError("f_new and f_old must have the same shape")
        self._check(self.lib.bt_set_schedule(self.h, _dp(fn), _dp(fo), fn.shape[1], fn.shape[0],
                                             float(dt), float(theta)))

    def set_schedule_phase(self, F_old):
        """F(tp) at the explicit level of every step, [n_sequences][n_steps] (the
        phase of the pseudo-periodic boundary term)."""
        Fo = np.ascontiguousarray(np.atleast_2d(np.asarray(F_old, np.float64)))
        self._check(self.lib.bt_set_schedule_phase(self.h, _dp(Fo), Fo.shape[1], Fo.shape[0]))

    def set_schedule_integral(self, F_new, F_old):
        """ift = int_0^t f at the implicit (F_new) and explicit (F_old) level of
        every step, [n_sequences][n_steps]: the strong pseudo-periodic form's
        schedule (also the weak form's phase)."""
        Fn = np.ascontiguousarray(np.atleast_2d(np.asarray(F_new, np.float64)))
        Fo = np.ascontiguousarray(np.atleast_2d(np.asarray(F_old, np.float64)))
        if Fn.shape != Fo.shape:
            raise ValueError("F_new and F_old must have the same shape")
        self._check(self.lib.bt_set_schedule_integral(self.h, _dp(Fn), _dp(Fo), Fn.shape[1], Fn.shape[0]))

    def set_periodic_mode(self, mode):
        """'weak' (IsDomainPeriodic = False, the default) or 'strong'
        (IsDomainPeriodic = True: constrained periodic space, FP64 BiCGSTAB)."""
        self._check(self.lib.bt_set_periodic_mode(self.h, {"weak": 0, "strong": 1}[mode]))

    def strong_periodic_info(self):
        n, nnz, ncl = C.c_int64(0), C.c_int64(0), C.c_int64(0)
        self._check(self.lib.bt_strong_periodic_info(self.h, C.byref(n), C.byref(nnz), C.byref(ncl)))
        return {"n_dofs": n.value, "nnz": nnz.value, "n_classes": ncl.value}

    def set_periodic(self, periodic_dir):
        """Pseudo-periodic boundaries along the axes with periodic_dir[d] = 1 in
        the form set_periodic_mode selected (weak by default; None or [0, 0, 0]
        switches them off)."""
        d = None if periodic_dir is None else np.ascontiguousarray(np.asarray(periodic_dir, np.int32).reshape(3))
        self._check(self.lib.bt_set_periodic(self.h, None if d is None else d.ctypes.data_as(_I32)))

    def periodic_info(self):
        pi = PeriodicInfo()
        self._check(self.lib.bt_periodic_info(self.h, C.byref(pi)))
        out = {k: getattr(pi, k) for k, _ in pi._fields_}
        out["dir"] = list(pi.dir)
        return out

    def solve(self, q, gdir, sequence=None, u0=None, precision=PRECISION_FP64, rtol=1e-12,
              max_iterations=2000, compartments=False):
        q = np.ascontiguousarray(np.atleast_1d(np.asarray(q, np.float64)))
        n = len(q)
        g = np.ascontiguousarray(np.asarray(gdir, np.float64).reshape(n, 3))
        seq = None if sequence is None else np.ascontiguousarray(np.asarray(sequence, np.int32).reshape(n))
        u = None if u0 is None else np.ascontiguousarray(np.asarray(u0, np.float64).reshape(self.n_vertices))
        sig = np.zeros(n)
        comp = np.zeros(n * self.n_compartments) if compartments else None
        S0 = C.c_double(0.0)
        st = Stats()
        self._check(self.lib.bt_solve(self.h, n, _dp(q), _dp(g), _ip(seq), _dp(u), int(precision),
                                      float(rtol), int(max_iterations), _dp(sig), _dp(comp),
                                      C.byref(S0), C.byref(st)))
        out = {"signal": sig, "S0": S0.value, "stats": st.as_dict()}
        if compartments:
            out["compartments"] = comp.reshape(n, self.n_compartments)
        return out

    def adjoint(self, q, gdir, sequence=0, u0=None, rtol=1e-13, max_iterations=5000, stride=0):
        """Signal and its derivatives (unnormalised) w.r.t. per-region D, 1/T2
        and pair permeabilities, by the discrete adjoint of the FP64 solve."""
        g = np.ascontiguousarray(np.asarray(gdir, np.float64).reshape(3))
        u = None if u0 is None else np.ascontiguousarray(np.asarray(u0, np.float64).reshape(self.n_vertices))
        nr = self.n_regions
        sig = np.zeros(1)
        dD, dT = np.zeros(nr), np.zeros(nr)
        dK = np.zeros(nr * nr)
        st = Stats()
        self._check(self.lib.bt_adjoint(self.h, float(q), _dp(g), int(sequence), _dp(u), float(rtol),
                                        int(max_iterations), int(stride), _dp(sig), _dp(dD), _dp(dT), _dp(dK),
                                        C.byref(st)))
        return {"signal": float(sig[0]), "dD": dD, "dinvT2": dT, "dkappa": dK.reshape(nr, nr),
                "stats": st.as_dict()}

    def solve_dev(self, q, gdir, sequence=None, u0=None, precision=PRECISION_FP64, rtol=1e-12, max_iterations=2000,
                  compartments=False):
        """bt_solve on device tensors: q[n], gdir[n, 3] (float64), sequence[n] (int32,
        optional), u0[n_vertices] (float64, optional), all CUDA tensors on this
        context's device; returns {"signal": tensor[n], "compartments": tensor[n, nc]
        or None, "S0": float, "stats": dict} with the tensors on the same device."""
        import torch

        def dev(t, dtype):
            if t is None:
                return None
            if not (torch.is_tensor(t) and t.is_cuda and t.dtype == dtype):
                raise TypeError("solve_dev takes CUDA tensors of dtype %s" % dtype)
            return t.contiguous()
        q = dev(q, torch.float64)
        n = q.numel()
        g = dev(gdir, torch.float64).reshape(n, 3).contiguous()
        seq = dev(sequence, torch.int32)
        u = dev(u0, torch.float64)
        sig = torch.empty(n, dtype=torch.float64, device=q.device)
        comp = torch.empty((n, self.n_compartments), dtype=torch.float64, device=q.device) if compartments else None
        S0 = C.c_double(0.0)
        st = Stats()
        ptr = (lambda t: None if t is None else C.c_void_p(t.data_ptr()))
        self._check(self.lib.bt_solve_dev(self.h, n, ptr(q), ptr(g), ptr(seq), ptr(u), int(precision), float(rtol),
                                          int(max_iterations), ptr(sig), ptr(comp), C.byref(S0), C.byref(st)))
        return {"signal": sig, "compartments": comp, "S0": S0.value, "stats": st.as_dict()}

    def adjoint_cells(self, q, gdir, sequence=0, u0=None, rtol=1e-13, max_iterations=5000, stride=0):
        """Signal and its derivatives (unnormalised) w.r.t. a per-cell diffusion
        tensor dD_cell[n_cells, 6] (xx, yy, zz, xy, xz, yz), a per-cell 1/T2
        dinvT2_cell[n_cells] and the pair permeabilities, by the FP64 adjoint."""
        g = np.ascontiguousarray(np.asarray(gdir, np.float64).reshape(3))
        u = None if u0 is None else np.ascontiguousarray(np.asarray(u0, np.float64).reshape(self.n_vertices))
        nr, nt = self.n_regions, self.info()["n_cells"]
        sig = np.zeros(1)
        d6, dT = np.zeros(nt * 6), np.zeros(nt)
        dK = np.zeros(nr * nr)
        st = Stats()
        self._check(self.lib.bt_adjoint_cells(self.h, float(q), _dp(g), int(sequence), _dp(u), float(rtol),
                                              int(max_iterations), int(stride), _dp(sig), _dp(d6), _dp(dT),
                                              _dp(dK), C.byref(st)))
        return {"signal": float(sig[0]), "dD_cell": d6.reshape(nt, 6), "dinvT2_cell": dT,
                "dkappa": dK.reshape(nr, nr), "stats": st.as_dict()}

    def adjoint_batch_cells(self, q, gdir, weights, sequence=None, rtol=1e-9, max_iterations=20000, stride=0):
        """Per-cell gradients of sum_s weights[s] S_s (unnormalised) by the batched
        mixed-precision adjoint: signal[n], dD_cell[n_cells, 6], dinvT2_cell[n_cells],
        dkappa[nr, nr]."""
        q = np.ascontiguousarray(np.atleast_1d(np.asarray(q, np.float64)))
        n = len(q)
        g = np.ascontiguousarray(np.asarray(gdir, np.float64).reshape(n, 3))
        w = np.ascontiguousarray(np.asarray(weights, np.float64).reshape(n))
        seq = None if sequence is None else np.ascontiguousarray(np.asarray(sequence, np.int32).reshape(n))
        nr, nt = self.n_regions, self.info()["n_cells"]
        sig = np.zeros(n)
        d6, dT, dK = np.zeros(nt * 6), np.zeros(nt), np.zeros(nr * nr)
        st = Stats()
        self._check(self.lib.bt_adjoint_batch_cells(self.h, n, _dp(q), _dp(g), _ip(seq), _dp(w), float(rtol),
                                                    int(max_iterations), int(stride), _dp(sig), _dp(d6), _dp(dT),
                                                    _dp(dK), C.byref(st)))
        return {"signal": sig, "dD_cell": d6.reshape(nt, 6), "dinvT2_cell": dT, "dkappa": dK.reshape(nr, nr),
                "stats": st.as_dict()}

    def adjoint_batch(self, q, gdir, sequence=None, rtol=1e-9, max_iterations=20000, stride=0):
        """The discrete adjoint of many signals at once in mixed precision:
        signal[n], dD[n, nr], dinvT2[n, nr], dkappa[n, nr, nr] (unnormalised)."""
        q = np.ascontiguousarray(np.atleast_1d(np.asarray(q, np.float64)))
        n = len(q)
        g = np.ascontiguousarray(np.asarray(gdir, np.float64).reshape(n, 3))
        seq = None if sequence is None else np.ascontiguousarray(np.asarray(sequence, np.int32).reshape(n))
        nr = self.n_regions
        sig = np.zeros(n)
        dD, dT, dK = np.zeros(n * nr), np.zeros(n * nr), np.zeros(n * nr * nr)
        st = Stats()
        self._check(self.lib.bt_adjoint_batch(self.h, n, _dp(q), _dp(g), _ip(seq), float(rtol), int(max_iterations),
                                              int(stride), _dp(sig), _dp(dD), _dp(dT), _dp(dK), C.byref(st)))
        return {"signal": sig, "dD": dD.reshape(n, nr), "dinvT2": dT.reshape(n, nr),
                "dkappa": dK.reshape(n, nr, nr), "stats": st.as_dict()}

    def tangent(self, q, gdir, param, i, j=0, sequence=0, u0=None, rtol=1e-13, max_iterations=5000):
        """Signal and d(signal)/d(param) by a tangent-linear FP64 run; param is
        "D" or "invT2" (region i) or "kappa" (region pair i, j)."""
        kinds = {"D": 0, "invT2": 1, "kappa": 2}
        g = np.ascontiguousarray(np.asarray(gdir, np.float64).reshape(3))
        u = None if u0 is None else np.ascontiguousarray(np.asarray(u0, np.float64).reshape(self.n_vertices))
        sig, d = np.zeros(1), np.zeros(1)
        st = Stats()
        self._check(self.lib.bt_tangent(self.h, float(q), _dp(g), int(sequence), _dp(u), kinds[param], int(i), int(j),
                                        float(rtol), int(max_iterations), _dp(sig), _dp(d), C.byref(st)))
        return {"signal": float(sig[0]), "d": float(d[0]), "stats": st.as_dict()}

    def csr(self):
        inf = self.info()
        rp = np.zeros(inf["n_dofs"] + 1, np.int32)
        col = np.zeros(inf["nnz"], np.int32)
        self._check(self.lib.bt_get_csr(self.h, _ip(rp), _ip(col)))
        return rp, col

    def matrix(self, which):
        inf = self.info()
        v = np.zeros(inf["nnz"])
        self._check(self.lib.bt_get_matrix(self.h, MATRICES[which], _dp(v)))
        return v

    def dofs(self):
        inf = self.info()
        dv = np.zeros(inf["n_dofs"], np.int32)
        dc = np.zeros(inf["n_dofs"], np.int32)
        w = np.zeros(inf["n_dofs"])
        self._check(self.lib.bt_get_dofs(self.h, _ip(dv), _ip(dc), _dp(w)))
        return dv, dc, w

    def colouring(self):
        c = np.zeros(self.info()["n_cells"], np.int32)
        self._check(self.lib.bt_get_colouring(self.h, _ip(c)))
        return c

    def solution(self, index=0):
        u = np.zeros(2 * self.info()["n_dofs"])
        self._check(self.lib.bt_get_solution(self.h, int(index), _dp(u)))
        return u[0::2] + 1j * u[1::2]

    def iterations(self, n_signals, n_steps):
        it = np.zeros(n_signals * n_steps, np.int32)
        self._check(self.lib.bt_get_iterations(self.h, _ip(it), it.size))
        return it.reshape(n_signals, n_steps)


def solve_multi(contexts, q, gdir, sequence=None, rtol=1e-9, max_iterations=5000):
    """Several meshes in one persistent mixed-precision launch.

    ``contexts[m]`` holds mesh m (uploaded, assembled, with a schedule);
    ``q[m]``, ``gdir[m]`` (and ``sequence[m]``) are that mesh's signals.
    Returns {"signal": [array per mesh], "S0": array, "stats": dict}."""
    nm = len(contexts)
    qs = [np.atleast_1d(np.asarray(x, np.float64)) for x in q]
    if len(qs) != nm or len(gdir) != nm:
        raise ValueError("one q list and one gdir list per context")
    nsig = np.ascontiguousarray([len(x) for x in qs], np.int32)
    qa = np.ascontiguousarray(np.concatenate(qs))
    ga = np.ascontiguousarray(np.concatenate([np.asarray(g, np.float64).reshape(len(x), 3)
                                              for g, x in zip(gdir, qs)]))
    sa = None if sequence is None else np.ascontiguousarray(
        np.concatenate([np.asarray(s_, np.int32).reshape(len(x)) for s_, x in zip(sequence, qs)]))
    handles = (_P * nm)(*[c.h for c in contexts])
    sig = np.zeros(len(qa))
    S0 = np.zeros(nm)
    st = Stats()
    lib = contexts[0].lib
    contexts[0]._check(lib.bt_solve_multi(handles, nm, _ip(nsig), _dp(qa), _dp(ga), _ip(sa), float(rtol),
                                          int(max_iterations), _dp(sig), _dp(S0), C.byref(st)))
    cuts = np.cumsum(nsig)[:-1]
    return {"signal": np.split(sig, cuts), "S0": S0, "stats": st.as_dict()}


def adjoint_multi(contexts, q, gdir, sequence=None, rtol=1e-9, max_iterations=20000, stride=0):
    """The batched mixed-precision adjoint of several meshes in one call.

    ``contexts[m]`` holds mesh m (uploaded, assembled, with a schedule);
    ``q[m]``, ``gdir[m]`` (and ``sequence[m]``) are that mesh's signals.  Returns
    per mesh the signals and the unnormalised gradients: {"signal": [n_m],
    "dD": [n_m x nr_m], "dinvT2": [n_m x nr_m], "dkappa": [n_m x nr_m x nr_m]}
    lists, and the stats."""
    nm = len(contexts)
    qs = [np.atleast_1d(np.asarray(x, np.float64)) for x in q]
    if len(qs) != nm or len(gdir) != nm:
        raise ValueError("one q list and one gdir list per context")
    nsig = np.ascontiguousarray([len(x) for x in qs], np.int32)
    qa = np.ascontiguousarray(np.concatenate(qs))
    ga = np.ascontiguousarray(np.concatenate([np.asarray(g, np.float64).reshape(len(x), 3)
                                              for g, x in zip(gdir, qs)]))
    sa = None if sequence is None else np.ascontiguousarray(
        np.concatenate([np.asarray(s_, np.int32).reshape(len(x)) for s_, x in zip(sequence, qs)]))
    nrs = [c.n_regions for c in contexts]
    nD = int(sum(n * r for n, r in zip(nsig, nrs)))
    nK = int(sum(n * r * r for n, r in zip(nsig, nrs)))
    handles = (_P * nm)(*[c.h for c in contexts])
    sig, dD, dT, dK = np.zeros(len(qa)), np.zeros(nD), np.zeros(nD), np.zeros(nK)
    st = Stats()
    lib = contexts[0].lib
    contexts[0]._check(lib.bt_adjoint_multi(handles, nm, _ip(nsig), _dp(qa), _dp(ga), _ip(sa), float(rtol),
                                            int(max_iterations), int(stride), _dp(sig), _dp(dD), _dp(dT), _dp(dK),
                                            C.byref(st)))
    out = {"signal": [], "dD": [], "dinvT2": [], "dkappa": [], "stats": st.as_dict()}
    a = b = c = 0
    for n, r in zip(nsig, nrs):
        out["signal"].append(sig[a:a + n])
        out["dD"].append(dD[b:b + n * r].reshape(n, r))
        out["dinvT2"].append(dT[b:b + n * r].reshape(n, r))
        out["dkappa"].append(dK[c:c + n * r * r].reshape(n, r, r))
        a, b, c = a + n, b + n * r, c + n * r * r
    return out
