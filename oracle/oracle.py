"""Python binding of the CPU oracle (TEST INFRASTRUCTURE ONLY).

Loaded by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg to check or time the
engine; the engine itself never imports this module.
"""
import ctypes as C
import os
import sys

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
from stablercwa_gb300 import abi  # noqa: E402  (struct layouts of the public C ABI)
from oracle import build as _build  # noqa: E402

_lib = None


def lib():
    global _lib
    if _lib is None:
        path = _build.build_oracle()
        L = C.CDLL(path)
        L.oracle_solve1d_batch.restype = C.c_int
        L.oracle_solve1d_batch.argtypes = [C.POINTER(abi.rcwa_stack1d), C.c_void_p, C.c_int, C.c_int, C.c_int,
                                           C.c_int, C.POINTER(abi.rcwa_result1d), C.c_int, C.c_char_p, C.c_size_t]
        L.oracle_solve_conical_batch.restype = C.c_int
        L.oracle_solve_conical_batch.argtypes = [C.POINTER(abi.rcwa_stack1d), C.c_void_p, C.c_int, C.c_int,
                                                 C.POINTER(abi.rcwa_result_conical), C.c_int, C.c_char_p, C.c_size_t]
        L.oracle_eig.argtypes = [C.c_int, C.c_void_p, C.c_double, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        L.oracle_schur.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        L.oracle_solve.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        L.oracle_multiply.argtypes = [C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
        L.oracle_eig_residual.restype = C.c_double
        L.oracle_eig_residual.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
        L.oracle_layer_matrix.argtypes = [C.POINTER(abi.rcwa_layer1d), C.c_double, C.c_double, C.c_double,
                                          C.c_double, C.c_int, C.c_int, C.c_void_p]
        L.oracle_layer_operators2d.restype = C.c_int
        L.oracle_layer_operators2d.argtypes = [C.POINTER(abi.rcwa_layer2d), C.c_double, C.c_double, C.c_int, C.c_int,
                                               C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
        L.oracle_solve2d_fields.restype = C.c_int
        L.oracle_solve2d_fields.argtypes = [C.POINTER(abi.rcwa_stack2d), C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int,
                                            C.c_void_p, C.c_int, C.POINTER(abi.rcwa_result2d), C.c_void_p, C.c_int,
                                            C.c_char_p, C.c_size_t]
        L.oracle_solve2d_batch.restype = C.c_int
        L.oracle_solve2d_batch.argtypes = [C.POINTER(abi.rcwa_stack2d), C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int,
                                           C.POINTER(abi.rcwa_result2d), C.c_int, C.c_char_p, C.c_size_t]
        _lib = L
    return _lib


class OracleInvalidArgument(ValueError):
    pass


def solve1d_batch(stack, points, M, pol, threads=1, diagnostics=False):
    """rcwa::sweep on the CPU: returns a dict of numpy arrays (R, T, DEr, DEt, status, ...)."""
    st, keep = abi.marshal_stack1d(stack)
    pts = abi.points_array(points)
    res, arrays = abi.result_views(len(pts), M)
    err = C.create_string_buffer(512)
    rc = lib().oracle_solve1d_batch(C.byref(st), pts.ctypes.data, len(pts), M, pol, 1 if diagnostics else 0,
                                    C.byref(res), threads, err, 512)
    if rc != 0:
        raise OracleInvalidArgument(err.value.decode())
    return arrays


def solve_conical_batch(stack, points, M, threads=1):
    """rcwa::sweep_conical on the CPU: dict of numpy arrays (Jr, Jt, DEr, DEt: (P, 2M+1, 4), ...)."""
    st, keep = abi.marshal_stack1d(stack)
    pts = abi.conical_points_array(points)
    res, arrays = abi.conical_views(len(pts), M)
    err = C.create_string_buffer(512)
    rc = lib().oracle_solve_conical_batch(C.byref(st), pts.ctypes.data, len(pts), M, C.byref(res), threads, err, 512)
    if rc != 0:
        raise OracleInvalidArgument(err.value.decode())
    return arrays


def eig(a, eps=2.220446049250313e-16, max_iter=30, vectors=True):
    a = np.asfortranarray(a, dtype=np.complex128)
    n = a.shape[0]
    w = np.empty(n, np.complex128)
    v = np.zeros((n, n), np.complex128, order="F") if vectors else None
    info = C.c_int()
    sweeps = C.c_int()
    lib().oracle_eig(n, a.ctypes.data, eps, max_iter, w.ctypes.data, v.ctypes.data if vectors else None,
                     C.byref(info), C.byref(sweeps))
    return w, v, info.value, sweeps.value


def schur(a):
    a = np.asfortranarray(a, dtype=np.complex128)
    n = a.shape[0]
    z = np.zeros((n, n), np.complex128, order="F")
    t = np.zeros((n, n), np.complex128, order="F")
    info = C.c_int()
    lib().oracle_schur(n, a.ctypes.data, z.ctypes.data, t.ctypes.data, C.byref(info))
    return z, t, info.value


def solve(a, b):
    a = np.asfortranarray(a, dtype=np.complex128)
    b = np.asfortranarray(b, dtype=np.complex128)
    n = a.shape[0]
    nrhs = b.shape[1]
    x = np.zeros((n, nrhs), np.complex128, order="F")
    sing = C.c_int()
    lib().oracle_solve(n, nrhs, a.ctypes.data, b.ctypes.data, x.ctypes.data, C.byref(sing))
    return x, bool(sing.value)


def multiply(a, b):
    a = np.asfortranarray(a, dtype=np.complex128)
    b = np.asfortranarray(b, dtype=np.complex128)
    c = np.zeros((a.shape[0], b.shape[1]), np.complex128, order="F")
    lib().oracle_multiply(a.shape[0], a.shape[1], b.shape[1], a.ctypes.data, b.ctypes.data, c.ctypes.data)
    return c


def eig_residual(a, values, vectors):
    a = np.asfortranarray(a, dtype=np.complex128)
    values = np.ascontiguousarray(values, dtype=np.complex128)
    vectors = np.asfortranarray(vectors, dtype=np.complex128)
    return lib().oracle_eig_residual(a.shape[0], a.ctypes.data, values.ctypes.data, vectors.ctypes.data)


def layer_matrix(layer, period, wavelength, nI, theta_deg, M, pol):
    class _S:  # marshal a one-layer stack to reuse the layer struct
        pass
    s = _S()
    s.nI, s.nII, s.period, s.layers = 1.0, 1.0, period, [layer]
    st, keep = abi.marshal_stack1d(s)
    n = 2 * M + 1
    a = np.zeros((n, n), np.complex128, order="F")
    rc = lib().oracle_layer_matrix(st.layers, period, wavelength, nI, theta_deg, M, pol, a.ctypes.data)
    if rc != 0:
        raise ArithmeticError("singular permittivity matrix")
    return a


def layer_operators2d(layer, Lx, Ly, M1, M2, laurent=False):
    """(Eps, Cx, Cy) of one 2-D layer as N x N arrays, and a singular flag (rcwa2d_operators.hpp:325-429)."""
    N = (2 * M1 + 1) * (2 * M2 + 1)
    keep = []
    L = abi.rcwa_layer2d()
    abi.marshal_layer2d(layer, L, keep)
    out = [np.zeros((N, N), np.complex128) for _ in range(3)]
    rc = lib().oracle_layer_operators2d(C.byref(L), Lx, Ly, M1, M2, 1 if laurent else 0,
                                        *[o.ctypes.data for o in out])
    return out[0], out[1], out[2], rc != 0


def solve2d_batch(stack, points, M1, M2, laurent=False, threads=1):
    """rcwa::solve2d per point on the CPU: dict of numpy arrays shaped (P, N) as abi.result2d_views gives
    (n_dense_solve is not restated). points: (wavelength, theta_deg, phi_deg, Es, Ep) tuples."""
    st, keep = abi.marshal_stack2d(stack)
    pts = abi.points2d_array(points)
    N = (2 * M1 + 1) * (2 * M2 + 1)
    res, arrays = abi.result2d_views(len(points), N, len(stack.layers))
    err = C.create_string_buffer(512)
    rc = lib().oracle_solve2d_batch(C.byref(st), C.cast(pts, C.c_void_p), len(points), M1, M2, 1 if laurent else 0,
                                    C.byref(res), threads, err, 512)
    if rc != 0:
        raise OracleInvalidArgument(err.value.decode())
    return arrays


def solve2d_fields(stack, points, M1, M2, zs, laurent=False, threads=1):
    """solve2d_batch plus the near-field harmonics at depths zs (include/stablercwa/rcwa2d_fields.hpp): returns
    (arrays, fields) with fields shaped (P, 6, N, len(zs)), components Ex, Ey, Ez, Hx, Hy, Hz."""
    st, keep = abi.marshal_stack2d(stack)
    pts = abi.points2d_array(points)
    N = (2 * M1 + 1) * (2 * M2 + 1)
    res, arrays = abi.result2d_views(len(points), N, len(stack.layers))
    z = np.ascontiguousarray(zs, np.float64)
    fields = np.zeros((len(points), 6, N, len(z)), np.complex128)
    err = C.create_string_buffer(512)
    rc = lib().oracle_solve2d_fields(C.byref(st), C.cast(pts, C.c_void_p), len(points), M1, M2, 1 if laurent else 0,
                                     z.ctypes.data, len(z), C.byref(res), fields.ctypes.data, threads, err, 512)
    if rc != 0:
        raise OracleInvalidArgument(err.value.decode())
    return arrays, fields
