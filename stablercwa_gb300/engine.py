"""Host-side mirror of StableRCWA's solve API over the engine's C ABI.

    from stablercwa_gb300 import Layer, Stack, TE
    from stablercwa_gb300.engine import Engine
    eng = Engine()
    r = eng.solve(stack, 1.053, 66.36, 20, TE)      # rcwa::solve (include/stablercwa/rcwa1d.hpp:1077)
    rs = eng.sweep(stack, points, 60, TE)            # rcwa::sweep (include/stablercwa/rcwa1d.hpp:1084)

Invalid arguments raise ValueError where the reference throws std::invalid_argument; numerical
failures give NaN results with a status, as the reference does. The compute path is
libstablercwa_gb300.so; there is no CPU fallback: without the library or a CUDA device the
constructor raises.
"""
import ctypes as C
import os

import numpy as np

from . import abi
from .types import Options, Result

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = os.path.join(_HERE, "_build", "libstablercwa_gb300.so")
_lib = None


class EngineError(RuntimeError):
    def __init__(self, code, message):
        super().__init__(f"rcwa_gb300 error {code}: {message}")
        self.code = code


class UnsupportedOption(EngineError):
    pass


def library_path():
    return _LIB


def load_library(build_if_missing=True):
    """Load libstablercwa_gb300.so (building it in-tree first if it is missing or stale)."""
    global _lib
    if _lib is not None:
        return _lib
    if build_if_missing:
        from . import build as _build
        _build.build()
    if not os.path.exists(_LIB):
        raise EngineError(abi.RCWA_ECUDA, f"{_LIB} is missing: run stablercwa_gb300/build.py")
    L = C.CDLL(_LIB)
    vp, ci, cd = C.c_void_p, C.c_int, C.c_double
    L.rcwa_gpu_create.argtypes = [C.POINTER(abi.rcwa_gpu_config), C.POINTER(vp)]
    L.rcwa_gpu_destroy.argtypes = [vp]
    L.rcwa_gpu_last_error.argtypes = [vp, C.c_char_p, C.c_size_t]
    L.rcwa_gpu_synchronize.argtypes = [vp]
    L.rcwa_gpu_launch_count.restype = C.c_longlong
    L.rcwa_gpu_stream.restype = vp
    L.rcwa_gpu_stream.argtypes = [vp]
    L.rcwa_gpu_set_kernel_timing.argtypes = [vp, ci]
    L.rcwa_gpu_kernel_time.argtypes = [vp, C.c_char_p, C.POINTER(cd), C.POINTER(C.c_longlong)]
    L.rcwa_gpu_kernel_busy.argtypes = [vp, C.c_char_p, C.POINTER(cd)]
    L.rcwa_options_default.argtypes = [C.POINTER(abi.rcwa_options)]
    L.rcwa_gpu_solve1d_batch.argtypes = [vp, C.POINTER(abi.rcwa_stack1d), vp, ci, ci, ci, C.POINTER(abi.rcwa_options),
                                         C.POINTER(abi.rcwa_result1d)]
    L.rcwa_gpu_solve1d_batch_dev.argtypes = L.rcwa_gpu_solve1d_batch.argtypes
    L.rcwa_gpu_solve1d_fields.argtypes = [vp, C.POINTER(abi.rcwa_stack1d), vp, ci, ci, ci, C.POINTER(abi.rcwa_options), vp,
                                          ci, C.POINTER(abi.rcwa_result1d), vp, vp]
    L.rcwa_gpu_solve_conical_batch.argtypes = [vp, C.POINTER(abi.rcwa_stack1d), vp, ci, ci,
                                               C.POINTER(abi.rcwa_options), C.POINTER(abi.rcwa_result_conical)]
    L.rcwa_gpu_solve_conical_fields.argtypes = [vp, C.POINTER(abi.rcwa_stack1d), vp, ci, ci, C.POINTER(abi.rcwa_options),
                                                vp, vp, ci, C.POINTER(abi.rcwa_result_conical), vp, vp]
    L.rcwa_gpu_solve2d_batch.argtypes = [vp, C.POINTER(abi.rcwa_stack2d), vp, ci, ci, ci, ci,
                                         C.POINTER(abi.rcwa_options), C.POINTER(abi.rcwa_result2d)]
    L.rcwa_gpu_solve2d_fields.argtypes = [vp, C.POINTER(abi.rcwa_stack2d), vp, ci, ci, ci, ci, C.POINTER(abi.rcwa_options),
                                          vp, ci, C.POINTER(abi.rcwa_result2d), vp]
    for name in ("rcwa_gpu_solve_json", "rcwa_gpu_server_solve_json"):
        getattr(L, name).argtypes = [vp, C.c_char_p, ci, C.POINTER(C.c_void_p), C.POINTER(ci)]
    L.rcwa_json_validate.argtypes = [C.c_char_p, ci, C.POINTER(C.c_void_p), C.POINTER(ci)]
    L.rcwa_fields_json_validate.argtypes = L.rcwa_json_validate.argtypes
    L.rcwa_gpu_solve_fields_json.argtypes = [vp, C.c_char_p, ci, C.POINTER(C.c_void_p), C.POINTER(ci)]
    L.rcwa_json_free.argtypes = [C.c_void_p]
    L.rcwa_gpu_field_slice.argtypes = [vp, vp, ci, ci, vp, vp, ci, ci, cd, cd, vp]
    L.rcwa_gpu_phase_data.argtypes = [vp, vp, ci, ci, ci, vp, vp, vp, vp, vp, cd, ci, vp, vp, vp, vp]
    L.rcwa_gpu_layer_operators2d.argtypes = [vp, C.POINTER(abi.rcwa_layer2d), cd, cd, ci, ci, ci, vp, vp, vp, vp]
    L.rcwa_gpu_server_create.argtypes = [C.POINTER(abi.rcwa_server_config), C.POINTER(vp)]
    L.rcwa_gpu_server_destroy.argtypes = [vp]
    L.rcwa_gpu_server_submit.argtypes = [vp, C.POINTER(abi.rcwa_request), C.POINTER(C.c_ulonglong)]
    L.rcwa_gpu_server_wait.argtypes = [vp, C.c_ulonglong, ci, C.POINTER(abi.rcwa_response), vp]
    L.rcwa_gpu_fourier_coefficients.argtypes = [vp, vp, vp, ci, cd, ci, ci, ci, vp]
    L.rcwa_gpu_eig_batch.argtypes = [vp, ci, ci, vp, cd, ci, vp, vp, vp, vp]
    L.rcwa_gpu_eig_batch_dev.argtypes = [vp, ci, ci, vp, cd, ci, vp, vp, vp, vp]
    L.rcwa_gpu_eig_hermitian_batch.argtypes = [vp, ci, ci, vp, cd, ci, vp, vp, vp]
    L.rcwa_gpu_eig_hermitian_batch_dev.argtypes = [vp, ci, ci, vp, cd, ci, vp, vp, vp]
    L.rcwa_gpu_solve_batch.argtypes = [vp, ci, ci, ci, vp, vp, vp, vp]
    L.rcwa_gpu_multiply_batch.argtypes = [vp, ci, ci, ci, ci, vp, vp, vp]
    L.rcwa_gpu_gemm_info.argtypes = [vp, vp, vp]
    L.rcwa_gpu_autotune_eig.argtypes = [vp, ci, ci, ci, vp, vp, vp]
    L.rcwa_gpu_autotune_set.argtypes = [ci, ci, ci, ci]
    L.rcwa_gpu_autotune_table.argtypes = [vp, C.c_size_t]
    _lib = L
    return L


def launch_count():
    return int(load_library().rcwa_gpu_launch_count())


def eig_rotations():
    """QL rotations of the Hermitian eigensolver since the previous call (resets the count)."""
    L = load_library()
    L.rcwa_gpu_eig_rotations.restype = C.c_longlong
    return int(L.rcwa_gpu_eig_rotations())


def _options(opt):
    o = abi.rcwa_options()
    load_library().rcwa_options_default(C.byref(o))
    if opt is not None:
        o.homogeneous_fast_path = 1 if opt.homogeneous_fast_path else 0
        o.diagnostics = 1 if opt.diagnostics else 0
        o.eig_max_iter = int(opt.eig_max_iter)
        o.eig_eps = float(opt.eig_eps)
    return o


def _colmajor(a):
    """(batch, n, m) row-indexed arrays -> column-major per matrix (contiguous)."""
    a = np.asarray(a, dtype=np.complex128)
    return np.ascontiguousarray(a.transpose(0, 2, 1))


class Engine:
    """One engine context on one CUDA device (rcwa_gpu_create / rcwa_gpu_destroy)."""

    def __init__(self, device=0, workspace_limit=0):
        self.L = load_library()
        cfg = abi.rcwa_gpu_config(device, workspace_limit)
        h = C.c_void_p()
        rc = self.L.rcwa_gpu_create(C.byref(cfg), C.byref(h))
        if rc != 0:
            raise EngineError(rc, self._err(None))
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.L.rcwa_gpu_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _err(self, h):
        buf = C.create_string_buffer(1024)
        self.L.rcwa_gpu_last_error(h, buf, 1024)
        return buf.value.decode(errors="replace")

    def _check(self, rc):
        if rc == abi.RCWA_EINVAL:
            raise ValueError(self._err(self.h))
        if rc == abi.RCWA_EUNSUPPORTED:
            raise UnsupportedOption(rc, self._err(self.h))
        if rc != 0:
            raise EngineError(rc, self._err(self.h))

    # ---------------------------------------------------------------- 1-D solve

    def solve1d_arrays(self, stack, points, M, pol, options=None):
        """Batched solve with host buffers; returns a dict of numpy arrays (R, T, DEr, DEt, status,
        eig_info, n_eig, n_dense_solve (the reference's count), max_eig_residual, n_lu (the engine's own LU
        factorisations per point)). pol = 2 (RCWA_TE_TM): both polarizations,
        every array holding the TE rows then the TM rows (2 x points)."""
        st, keep = abi.marshal_stack1d(stack)
        pts = abi.points_array(points)
        res, arrays = abi.result_views(len(pts) * (2 if pol == abi.RCWA_TE_TM else 1), M)
        o = _options(options)
        self._check(self.L.rcwa_gpu_solve1d_batch(self.h, C.byref(st), pts.ctypes.data, len(pts), M, pol, C.byref(o),
                                                  C.byref(res)))
        return arrays

    def solve1d_fields(self, stack, points, M, pol, zs, options=None):
        """rcwa::solve_with_fields + field_at at every point: (result arrays, fields) with fields of shape
        (points, 6, 2M+1, nz), components Ex, Ey, Ez, Hx, Hy, Hz (H = Z0 H), harmonics per order and depth."""
        st, keep = abi.marshal_stack1d(stack)
        pts = abi.points_array(points)
        z = np.ascontiguousarray(np.asarray(zs, dtype=np.float64).reshape(-1))
        res, arrays = abi.result_views(len(pts), M)
        fields = np.empty((len(pts), 6, 2 * M + 1, len(z)), np.complex128)
        info = np.zeros((len(pts), max(1, len(stack.layers))), np.int32)
        o = _options(options)
        self._check(self.L.rcwa_gpu_solve1d_fields(self.h, C.byref(st), pts.ctypes.data, len(pts), M, pol, C.byref(o),
                                                   z.ctypes.data, len(z), C.byref(res), fields.ctypes.data,
                                                   info.ctypes.data))
        arrays["layer_info"] = info
        return arrays, fields

    def solve_json(self, request, indent=-1):
        """rcwa::solve_json_reply (include/stablercwa/rcwa_json.hpp:1287-1309) on this context, every point
        of the request in one batched call: (ok, reply text)."""
        return _json_call(self.L.rcwa_gpu_solve_json, self.h, request, indent)

    def solve_fields_json(self, request, indent=-1):
        """rcwa::solve_fields_json_reply (include/stablercwa/rcwa_fields_json.hpp): one point with its fields,
        NPY files published into the request's output_dir; (ok, reply text)."""
        return _json_call(self.L.rcwa_gpu_solve_fields_json, self.h, request, indent)

    def field_slice(self, fields, kx, ky, plane, nt, period, at=0.0):
        """Real-space slice of one point's harmonics on the device (rcwa::field_slice, reconstruct_field_slice,
        rcwa_fields.hpp:357-385): fields (6, n, nz), kx and ky the physical wavevector of each harmonic (ky a
        scalar for a 1-D solve), plane abi.RCWA_SLICE_XZ (y = at) or RCWA_SLICE_YZ (x = at); returns
        (6, nz, nt) at t = (it / nt) period."""
        h = np.ascontiguousarray(fields, dtype=np.complex128)
        n, nz = h.shape[1], h.shape[2]
        kxa = np.ascontiguousarray(np.broadcast_to(np.asarray(kx, dtype=np.float64), (n,)))
        kya = np.ascontiguousarray(np.broadcast_to(np.asarray(ky, dtype=np.float64), (n,)))
        out = np.empty((6, nz, int(nt)), np.complex128)
        self._check(self.L.rcwa_gpu_field_slice(self.h, h.ctypes.data, n, nz, kxa.ctypes.data, kya.ctypes.data, int(plane),
                                                int(nt), float(period), float(at), out.ctypes.data))
        return out

    def field_map(self, fields, kxm, period, nx=256, y=0.0, ky=0.0):
        """The x-z map of rcwa::field_map (reconstruct_field_grid, rcwa_fields.hpp:326-355) on the device:
        fields (6, n, nz) of one point, kxm the physical kx of each order, ky the physical ky (0 for a planar
        solve, k0 ky for a conical one); returns (6, nz, nx)."""
        return self.field_slice(fields, kxm, ky, abi.RCWA_SLICE_XZ, nx, period, y)

    def phase_data(self, field, reference="absolute", phase_floor=1e-6, unwrap="none", incident_k=None, x=None, y=None,
                   z=None, custom=None):
        """rcwa::phase_data of one complex grid (nz, nt) on the device (rcwa_phase.hpp:229-271): dict of phase
        (NaN where masked), amplitude, mask and reference, each (nz, nt). reference: "absolute", "incident"
        (incident_k = (kx0, ky0, kz0) and the grid coordinates x, y (nt) and z (nz)) or "custom" (custom
        broadcast to the grid like numpy). unwrap: "none", "x", "z" or "both"."""
        f = np.ascontiguousarray(field, dtype=np.complex128)
        nz, nt = f.shape
        kinds = {"absolute": abi.RCWA_PHASE_ABSOLUTE, "incident": abi.RCWA_PHASE_INCIDENT, "custom": abi.RCWA_PHASE_CUSTOM}
        axes = {"none": abi.RCWA_UNWRAP_NONE, "x": abi.RCWA_UNWRAP_X, "t": abi.RCWA_UNWRAP_X, "horizontal": abi.RCWA_UNWRAP_X,
                "z": abi.RCWA_UNWRAP_Z, "vertical": abi.RCWA_UNWRAP_Z, "both": abi.RCWA_UNWRAP_BOTH}
        kind = kinds[reference] if isinstance(reference, str) else int(reference)
        ax = axes[unwrap] if isinstance(unwrap, str) else int(unwrap)
        keep = []

        def arr(v, dtype, shape=None):
            if v is None:
                return None
            a = np.asarray(v, dtype=dtype)
            if shape is not None:
                a = np.broadcast_to(a, shape)
            a = np.ascontiguousarray(a)
            keep.append(a)
            return a.ctypes.data
        out = {"phase": np.empty((nz, nt)), "amplitude": np.empty((nz, nt)), "mask": np.empty((nz, nt), np.uint8),
               "reference": np.empty((nz, nt), np.complex128)}
        self._check(self.L.rcwa_gpu_phase_data(
            self.h, f.ctypes.data, nt, nz, kind, arr(incident_k, np.float64), arr(x, np.float64), arr(y, np.float64),
            arr(z, np.float64), arr(custom, np.complex128, (nz, nt)) if custom is not None else None, float(phase_floor), ax,
            out["phase"].ctypes.data, out["amplitude"].ctypes.data, out["mask"].ctypes.data,
            out["reference"].ctypes.data if kind != abi.RCWA_PHASE_ABSOLUTE else None))
        out["mask"] = out["mask"].astype(bool)
        if kind == abi.RCWA_PHASE_ABSOLUTE:
            out["reference"] = None
        return out

    def solve1d_device(self, stack, d_points, n_points, M, pol, d_out, options=None):
        """Batched solve on device memory. d_points: device address of n_points (wavelength, theta)
        double pairs; d_out: dict of device addresses for R, T, DEr, DEt, status (others optional).
        pol = 2 (RCWA_TE_TM) solves both polarizations: every array holds TE results then TM results."""
        st, keep = abi.marshal_stack1d(stack)
        res = abi.rcwa_result1d()
        for k in ("R", "T", "DEr", "DEt", "status", "eig_info", "n_eig", "n_dense_solve", "max_eig_residual", "n_lu"):
            setattr(res, k, d_out.get(k))
        o = _options(options)
        self._check(self.L.rcwa_gpu_solve1d_batch_dev(self.h, C.byref(st), d_points, n_points, M, pol, C.byref(o),
                                                      C.byref(res)))

    def stream(self):
        """The context's cudaStream_t as an integer (torch.cuda.ExternalStream accepts it)."""
        return int(self.L.rcwa_gpu_stream(self.h) or 0)

    def set_kernel_timing(self, enable):
        self._check(self.L.rcwa_gpu_set_kernel_timing(self.h, 1 if enable else 0))

    def kernel_time(self, kind):
        """(milliseconds, launches) accumulated for 'eig', 'lu' or 'gemm' since the last read."""
        ms = C.c_double()
        n = C.c_longlong()
        self._check(self.L.rcwa_gpu_kernel_time(self.h, kind.encode(), C.byref(ms), C.byref(n)))
        return ms.value, n.value

    def kernel_busy(self, kind):
        """Milliseconds during which at least one 'eig' / 'lu' / 'gemm' launch was running, since the
        last read (launches of the two polarizations of a RCWA_TE_TM call overlap)."""
        ms = C.c_double()
        self._check(self.L.rcwa_gpu_kernel_busy(self.h, kind.encode(), C.byref(ms)))
        return ms.value

    def synchronize(self):
        self._check(self.L.rcwa_gpu_synchronize(self.h))

    def sweep(self, stack, points, M, pol, options=None):
        a = self.solve1d_arrays(stack, points, M, pol, options)
        orders = np.arange(-M, M + 1)
        return [Result(orders=orders, R=a["R"][p], T=a["T"][p], DEr=a["DEr"][p], DEt=a["DEt"][p],
                       eig_info=int(a["eig_info"][p]), n_eig=int(a["n_eig"][p]),
                       n_dense_solve=int(a["n_dense_solve"][p]), status=int(a["status"][p]),
                       max_eig_residual=float(a["max_eig_residual"][p]), n_lu=int(a["n_lu"][p]))
                for p in range(len(a["status"]))]

    def solve(self, stack, wavelength, theta_deg, M, pol=0, options=None):
        return self.sweep(stack, [(wavelength, theta_deg)], M, pol, options)[0]

    # ---------------------------------------------------------------- conical incidence

    def solve_conical_arrays(self, stack, points, M, options=None):
        """rcwa::sweep_conical over (wavelength, theta, phi) points: dict of numpy arrays with Jr, Jt
        (P, 2M+1, 4 complex: ss, sp, ps, pp), DEr, DEt (P, 2M+1, 4), status, eig_info, n_eig,
        n_dense_solve, n_schur, min_abs_lambda, degenerate_mode_warning, kx, ky, flux_r, flux_t, n_lu."""
        st, keep = abi.marshal_stack1d(stack)
        pts = abi.conical_points_array(points)
        res, arrays = abi.conical_views(len(pts), M)
        o = _options(options)
        self._check(self.L.rcwa_gpu_solve_conical_batch(self.h, C.byref(st), pts.ctypes.data, len(pts), M, C.byref(o),
                                                        C.byref(res)))
        return arrays

    def solve_conical_fields(self, stack, points, M, zs, jones=None, options=None):
        """rcwa::solve_conical_with_fields + field_at(context, zs, jones) at every (wavelength, theta, phi)
        point: (result arrays, fields (P, 6, 2M+1, nz)). jones: None for (1, 0), one (Es, Ep) pair for
        every point, or one pair per point; normalised like rcwa::normalized_jones."""
        st, keep = abi.marshal_stack1d(stack)
        pts = abi.conical_points_array(points)
        res, arrays = abi.conical_views(len(pts), M)
        z = np.ascontiguousarray(np.asarray(zs, dtype=np.float64).reshape(-1))
        fields = np.empty((len(pts), 6, 2 * M + 1, len(z)), np.complex128)
        jp = None
        if jones is not None:
            j = np.asarray(jones, dtype=np.complex128)
            j = np.ascontiguousarray(np.broadcast_to(j.reshape(-1, 2), (len(pts), 2)))
            jp = j.ctypes.data
        o = _options(options)
        info = np.zeros((len(pts), max(1, len(stack.layers))), np.int32)
        self._check(self.L.rcwa_gpu_solve_conical_fields(self.h, C.byref(st), pts.ctypes.data, len(pts), M, C.byref(o),
                                                         jp, z.ctypes.data, len(z), C.byref(res), fields.ctypes.data,
                                                         info.ctypes.data))
        arrays["layer_info"] = info
        return arrays, fields

    def solve_conical(self, stack, wavelength, theta_deg, phi_deg, M, options=None):
        a = self.solve_conical_arrays(stack, [(wavelength, theta_deg, phi_deg)], M, options)
        return {k: v[0] for k, v in a.items()}

    # ---------------------------------------------------------------- 2-D crossed gratings

    def solve2d_arrays(self, stack, points, M1, M2, laurent=False, options=None):
        """rcwa::solve2d at every (wavelength, theta_deg, phi_deg, Es, Ep) point: dict of numpy arrays
        (P, N) for Kx, Ky, kzI, kzII, Ex_r .. Ez_t, Rs, Rp, Ts, Tp, DEr, DEt, prop_r, prop_t and (P,)
        for status, eig_info, n_eig, n_dense_solve, max_eig_residual, plus rayleigh_regions
        (P, n_layers + 2)."""
        st, keep = abi.marshal_stack2d(stack)
        pts = abi.points2d_array(points)
        N = (2 * M1 + 1) * (2 * M2 + 1)
        res, arrays = abi.result2d_views(len(points), N, len(stack.layers))
        o = _options(options)
        fact = abi.RCWA_FACTORIZATION_LAURENT if laurent else abi.RCWA_FACTORIZATION_LI
        self._check(self.L.rcwa_gpu_solve2d_batch(self.h, C.byref(st), C.cast(pts, C.c_void_p), len(points), M1, M2,
                                                  fact, C.byref(o), C.byref(res)))
        return arrays

    def solve2d_fields(self, stack, points, M1, M2, zs, laurent=False, options=None):
        """rcwa::solve2d_with_fields + field_at(result, zs) at every (wavelength, theta_deg, phi_deg, Es, Ep)
        point: (result arrays, fields (P, 6, N, nz)), N = (2 M1 + 1)(2 M2 + 1)."""
        st, keep = abi.marshal_stack2d(stack)
        pts = abi.points2d_array(points)
        N = (2 * M1 + 1) * (2 * M2 + 1)
        res, arrays = abi.result2d_views(len(points), N, len(stack.layers))
        z = np.ascontiguousarray(np.asarray(zs, dtype=np.float64).reshape(-1))
        fields = np.empty((len(points), 6, N, len(z)), np.complex128)
        o = _options(options)
        fact = abi.RCWA_FACTORIZATION_LAURENT if laurent else abi.RCWA_FACTORIZATION_LI
        self._check(self.L.rcwa_gpu_solve2d_fields(self.h, C.byref(st), C.cast(pts, C.c_void_p), len(points), M1, M2, fact,
                                                   C.byref(o), z.ctypes.data, len(z), C.byref(res), fields.ctypes.data))
        return arrays, fields

    def solve2d(self, stack, wavelength, theta_deg, phi_deg, M1, M2, jones, laurent=False, options=None):
        """One rcwa::solve2d (include/stablercwa/rcwa2d.hpp:1359): arrays of that point, plus the
        reference's message for a Rayleigh anomaly (region and (m, n) list)."""
        a = self.solve2d_arrays(stack, [(wavelength, theta_deg, phi_deg, jones[0], jones[1])], M1, M2, laurent, options)
        r = {k: v[0] for k, v in a.items()}
        r["message"] = rayleigh_message(stack, r, M1, M2) if r["status"] == abi.RCWA_SAMPLE_RAYLEIGH else ""
        return r

    def layer_operators2d(self, layer, Lx, Ly, M1, M2, laurent=False):
        """Eps, Cx, Cy (N x N) of one layer (rcwa::detail2d::layer_operators,
        include/stablercwa/rcwa2d_operators.hpp:325) and the singular flag."""
        keep = []
        s = abi.rcwa_layer2d()
        abi.marshal_layer2d(layer, s, keep)
        N = (2 * M1 + 1) * (2 * M2 + 1)
        mats = [np.empty((N, N), np.complex128) for _ in range(3)]  # column-major storage: transposed below
        sing = C.c_int(0)
        fact = abi.RCWA_FACTORIZATION_LAURENT if laurent else abi.RCWA_FACTORIZATION_LI
        self._check(self.L.rcwa_gpu_layer_operators2d(self.h, C.byref(s), float(Lx), float(Ly), M1, M2, fact,
                                                      mats[0].ctypes.data, mats[1].ctypes.data, mats[2].ctypes.data,
                                                      C.byref(sing)))
        return mats[0].T.copy(), mats[1].T.copy(), mats[2].T.copy(), bool(sing.value)

    def fourier_coefficients(self, edges, values, period, hmax, method=0, samples=0):
        """c[h + hmax], h = -hmax..hmax: closed form (method 0, rcwa::detail::fourier_coefficients) or
        FFT-sampled with `samples` samples (method 1, rcwa::fourier_coefficients_fft)."""
        e = np.ascontiguousarray(np.asarray(edges, dtype=np.float64))
        v = np.ascontiguousarray(np.asarray(values, dtype=np.complex128))
        out = np.empty(2 * hmax + 1, np.complex128)
        self._check(self.L.rcwa_gpu_fourier_coefficients(self.h, e.ctypes.data, v.ctypes.data, len(v), float(period), hmax,
                                                         method, samples, out.ctypes.data))
        return out

    # ---------------------------------------------------------------- dense kernels (custom_* hooks)

    def eig_batch(self, a, eps=float(np.finfo(np.float64).eps), max_iter=30):
        """a: (batch, n, n). Returns values (batch, n), vectors (batch, n, n) with columns the
        eigenvectors, info (batch,), sweeps (batch,)."""
        a = np.asarray(a, dtype=np.complex128)
        batch, n = a.shape[0], a.shape[1]
        cm = _colmajor(a)
        w = np.empty((batch, n), np.complex128)
        v = np.empty((batch, n, n), np.complex128)
        info = np.empty(batch, np.int32)
        sweeps = np.empty(batch, np.int32)
        self._check(self.L.rcwa_gpu_eig_batch(self.h, n, batch, cm.ctypes.data, eps, max_iter, w.ctypes.data,
                                              v.ctypes.data, info.ctypes.data, sweeps.ctypes.data))
        return w, v.transpose(0, 2, 1), info, sweeps

    def eig_batch_device(self, n, batch, d_a, d_w, d_v, d_info, d_sweeps=None, eps=float(np.finfo(np.float64).eps),
                         max_iter=30):
        self._check(self.L.rcwa_gpu_eig_batch_dev(self.h, n, batch, d_a, eps, max_iter, d_w, d_v, d_info, d_sweeps))

    def autotune_eig(self, n, batch, d_a, hermitian=False):
        """Time every eigensolver form on `batch` device matrices at d_a and record the fastest
        (rcwa_gpu_autotune_eig): (form, milliseconds)."""
        form, ms = C.c_int(), C.c_double()
        self._check(self.L.rcwa_gpu_autotune_eig(self.h, 1 if hermitian else 0, n, batch, d_a, C.byref(form), C.byref(ms)))
        return form.value, ms.value

    def eig_hermitian_batch(self, a, eps=float(np.finfo(np.float64).eps), max_iter=30):
        """Hermitian part of a: (batch, n, n). Returns values (batch, n) real, unsorted; vectors (batch, n, n)
        with orthonormal columns; info (batch,)."""
        a = np.asarray(a, dtype=np.complex128)
        batch, n = a.shape[0], a.shape[1]
        cm = _colmajor(a)
        w = np.empty((batch, n), np.complex128)
        v = np.empty((batch, n, n), np.complex128)
        info = np.empty(batch, np.int32)
        self._check(self.L.rcwa_gpu_eig_hermitian_batch(self.h, n, batch, cm.ctypes.data, eps, max_iter, w.ctypes.data,
                                                        v.ctypes.data, info.ctypes.data))
        return w.real.copy(), v.transpose(0, 2, 1), info

    def eig_hermitian_batch_device(self, n, batch, d_a, d_w, d_v, d_info, eps=float(np.finfo(np.float64).eps),
                                   max_iter=30):
        self._check(self.L.rcwa_gpu_eig_hermitian_batch_dev(self.h, n, batch, d_a, eps, max_iter, d_w, d_v, d_info))

    def solve_batch(self, a, b):
        """Solve a[k] x[k] = b[k]; a: (batch, n, n), b: (batch, n, nrhs). Returns x, singular."""
        a = np.asarray(a, dtype=np.complex128)
        b = np.asarray(b, dtype=np.complex128)
        batch, n, nrhs = b.shape
        ca, cb = _colmajor(a), _colmajor(b)
        x = np.empty((batch, nrhs, n), np.complex128)
        sing = np.zeros(batch, np.int32)
        self._check(self.L.rcwa_gpu_solve_batch(self.h, n, nrhs, batch, ca.ctypes.data, cb.ctypes.data, x.ctypes.data,
                                                sing.ctypes.data))
        return x.transpose(0, 2, 1), sing.astype(bool)

    def multiply_batch(self, a, b):
        a = np.asarray(a, dtype=np.complex128)
        b = np.asarray(b, dtype=np.complex128)
        batch, m, k = a.shape
        n = b.shape[2]
        ca, cb = _colmajor(a), _colmajor(b)
        c = np.empty((batch, n, m), np.complex128)
        self._check(self.L.rcwa_gpu_multiply_batch(self.h, m, k, n, batch, ca.ctypes.data, cb.ctypes.data, c.ctypes.data))
        return c.transpose(0, 2, 1)


def autotune_set(hermitian, n, batch, form):
    """Record an eigensolver form for (solver, order, batch bucket) (rcwa_gpu_autotune_set); returns the code."""
    return load_library().rcwa_gpu_autotune_set(1 if hermitian else 0, n, batch, form)


def autotune_table():
    """The autotuner's table as text lines "<general|hermitian> <order> <batch bucket> <form>"."""
    L = load_library()
    size = L.rcwa_gpu_autotune_table(None, 0)
    buf = C.create_string_buffer(max(1, size + 1))
    L.rcwa_gpu_autotune_table(buf, len(buf))
    return buf.value.decode()


def gemm_info():
    """(tensor_cores, slices, stuck) of the engine's complex products (rcwa_gpu_gemm_info)."""
    L = load_library()
    t, sl, st = C.c_int(), C.c_int(), C.c_int()
    rc = L.rcwa_gpu_gemm_info(C.byref(t), C.byref(sl), C.byref(st))
    if rc != 0:
        raise EngineError(rc, "rcwa_gpu_gemm_info failed")
    return bool(t.value), sl.value, st.value


def _json_call(fn, handle, request, indent):
    L = load_library()
    out = C.c_void_p()
    ok = C.c_int(0)
    args = ([handle] if handle is not None else []) + [request.encode("utf-8"), int(indent), C.byref(out), C.byref(ok)]
    rc = fn(*args)
    if rc != 0:
        raise EngineError(rc, "JSON front end failed")
    try:
        text = C.cast(out, C.c_char_p).value.decode("utf-8")
    finally:
        L.rcwa_json_free(out)
    return bool(ok.value), text


def json_validate(request, indent=-1):
    """Checks a JSON request like the reference's reader (rcwa_json.hpp:739-800) without solving it:
    (True, "") when it is valid, else (False, the reference's error reply). Needs no GPU."""
    return _json_call(load_library().rcwa_json_validate, None, request, indent)


def fields_json_validate(request, indent=-1):
    """The request checks of the near-field protocol (rcwa_fields_json.hpp:68-151) alone: (True, "") or
    (False, the error reply). Needs no GPU."""
    return _json_call(load_library().rcwa_fields_json_validate, None, request, indent)


def rayleigh_message(stack, r, M1, M2):
    """Regions and (m, n) orders with kz exactly 0, listed as the reference lists them
    (report_rayleigh, include/stablercwa/rcwa2d.hpp:1012-1026), in English."""
    n2 = 2 * M2 + 1
    N = (2 * M1 + 1) * n2
    mn = [(i // n2 - M1, i % n2 - M2) for i in range(N)]
    parts = []

    def region(name, kz):
        orders = [mn[i] for i in range(N) if kz[i] == 0]
        if orders:
            parts.append(f"{name}: " + ", ".join(f"({m}, {n})" for m, n in orders))

    region("incident medium", r["kzI"])
    region("exit medium", r["kzII"])
    for j, L in enumerate(stack.layers):
        if L.homogeneous and r["rayleigh_regions"][j + 1]:
            nn = complex(L.n)
            kz = np.sqrt(nn * nn - r["Kx"] ** 2 - r["Ky"] ** 2)
            region(f"layer {j + 1}", kz)
    return "; ".join(parts)


class Server:
    """The serving request loop (rcwa_gpu_server_*): submit single solves of any kind, collect them
    with wait(). Requests run concurrently on `slots` worker slots, admitted by device footprint; queued
    requests of one structure (differing only in the point) share one batched call, up to `max_batch`
    (0: 256, 1: never)."""

    def __init__(self, device=0, slots=32, hbm_budget=0, max_bypass_ms=0, max_batch=0):
        self.L = load_library()
        cfg = abi.rcwa_server_config(device, slots, hbm_budget, max_bypass_ms, max_batch)
        h = C.c_void_p()
        rc = self.L.rcwa_gpu_server_create(C.byref(cfg), C.byref(h))
        if rc != 0:
            raise EngineError(rc, "rcwa_gpu_server_create failed")
        self.h = h
        self.meta = {}

    def close(self):
        if getattr(self, "h", None):
            self.L.rcwa_gpu_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def solve_json(self, request, indent=-1):
        """The JSON front end on the serving loop: one request per point, run on the worker slots; (ok, reply)."""
        return _json_call(self.L.rcwa_gpu_server_solve_json, self.h, request, indent)

    def _submit(self, req, meta):
        t = C.c_ulonglong()
        rc = self.L.rcwa_gpu_server_submit(self.h, C.byref(req), C.byref(t))
        if rc != 0:
            raise ValueError(f"rcwa_gpu_server_submit: error {rc}")
        self.meta[t.value] = meta
        return t.value

    def submit_1d(self, stack, wavelength, theta_deg, M, pol=0, options=None):
        st, keep = abi.marshal_stack1d(stack)
        req = abi.rcwa_request(kind=abi.RCWA_REQ_1D, stack1d=C.pointer(st), wavelength=wavelength, theta_deg=theta_deg,
                               M=M, polarization=pol, options=_options(options))
        return self._submit(req, ("1d", 2 * M + 1, 0))

    def submit_conical(self, stack, wavelength, theta_deg, phi_deg, M, options=None):
        st, keep = abi.marshal_stack1d(stack)
        req = abi.rcwa_request(kind=abi.RCWA_REQ_CONICAL, stack1d=C.pointer(st), wavelength=wavelength,
                               theta_deg=theta_deg, phi_deg=phi_deg, M=M, options=_options(options))
        return self._submit(req, ("conical", 2 * M + 1, 0))

    def submit_2d(self, stack, wavelength, theta_deg, phi_deg, M1, M2, jones, laurent=False, options=None):
        st, keep = abi.marshal_stack2d(stack)
        fact = abi.RCWA_FACTORIZATION_LAURENT if laurent else abi.RCWA_FACTORIZATION_LI
        req = abi.rcwa_request(kind=abi.RCWA_REQ_2D, stack2d=C.pointer(st), wavelength=wavelength, theta_deg=theta_deg,
                               phi_deg=phi_deg, M1=M1, M2=M2, factorization=fact, Es=abi.cplx(jones[0]),
                               Ep=abi.cplx(jones[1]), options=_options(options))
        return self._submit(req, ("2d", (2 * M1 + 1) * (2 * M2 + 1), len(stack.layers)))

    def wait(self, ticket, timeout_ms=-1):
        """(response dict, result arrays of the one point) or None on timeout."""
        kind, n, L = self.meta[ticket]
        if kind == "1d":
            res, arrays = abi.result_views(1, (n - 1) // 2)
        elif kind == "conical":
            res, arrays = abi.conical_views(1, (n - 1) // 2)
        else:
            res, arrays = abi.result2d_views(1, n, L)
        resp = abi.rcwa_response()
        rc = self.L.rcwa_gpu_server_wait(self.h, ticket, timeout_ms, C.byref(resp), C.cast(C.byref(res), C.c_void_p))
        if rc == abi.RCWA_ETIMEOUT:
            return None
        if rc == abi.RCWA_ECANCELLED:
            del self.meta[ticket]
            return {"code": rc, "kind": kind}, None
        if rc != 0:
            raise ValueError(f"rcwa_gpu_server_wait: error {rc}")
        del self.meta[ticket]
        r = {k: v[0] for k, v in arrays.items()}
        info = {"code": resp.code, "slot": resp.slot, "submit_s": resp.submit_s, "start_s": resp.start_s,
                "finish_s": resp.finish_s, "footprint_bytes": resp.footprint_bytes, "batch": resp.batch, "kind": kind}
        return info, r
