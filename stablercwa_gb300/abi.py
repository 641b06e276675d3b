"""ctypes mirror of the engine's C ABI (include/stablercwa_gb300.h).

The structs here are laid out exactly as the header declares them; marshal_stack1d turns the Python
Stack/Layer description into an rcwa_stack1d that stays valid while the returned keep-alive tuple
is referenced.
"""
import ctypes as C

import numpy as np

RCWA_OK = 0
RCWA_EINVAL = -1
RCWA_ECUDA = -2
RCWA_ENOMEM = -3
RCWA_EUNSUPPORTED = -4

RCWA_SAMPLE_OK = 0
RCWA_SAMPLE_NUMERICAL = 1
RCWA_SAMPLE_EIG_NOCONV = 2

RCWA_TE = 0
RCWA_TM = 1
RCWA_TE_TM = 2


class rcwa_complex(C.Structure):
    _fields_ = [("re", C.c_double), ("im", C.c_double)]


class rcwa_layer1d(C.Structure):
    _fields_ = [
        ("d", C.c_double),
        ("homogeneous", C.c_int),
        ("n", rcwa_complex),
        ("n_segments", C.c_int),
        ("edges", C.POINTER(C.c_double)),
        ("n_values", C.POINTER(rcwa_complex)),
        ("fourier_method", C.c_int),
        ("fft_samples", C.c_int),
    ]


class rcwa_stack1d(C.Structure):
    _fields_ = [
        ("nI", rcwa_complex),
        ("nII", rcwa_complex),
        ("period", C.c_double),
        ("n_layers", C.c_int),
        ("layers", C.POINTER(rcwa_layer1d)),
    ]


class rcwa_point1d(C.Structure):
    _fields_ = [("wavelength", C.c_double), ("theta_deg", C.c_double)]


class rcwa_options(C.Structure):
    _fields_ = [
        ("eig_method", C.c_int),
        ("linear_solver", C.c_int),
        ("homogeneous_fast_path", C.c_int),
        ("diagnostics", C.c_int),
        ("eig_max_iter", C.c_int),
        ("eig_eps", C.c_double),
    ]


class rcwa_result1d(C.Structure):
    _fields_ = [
        ("R", C.c_void_p),
        ("T", C.c_void_p),
        ("DEr", C.c_void_p),
        ("DEt", C.c_void_p),
        ("status", C.c_void_p),
        ("eig_info", C.c_void_p),
        ("n_eig", C.c_void_p),
        ("n_dense_solve", C.c_void_p),
        ("max_eig_residual", C.c_void_p),
        ("n_lu", C.c_void_p),
    ]


class rcwa_point_conical(C.Structure):
    _fields_ = [("wavelength", C.c_double), ("theta_deg", C.c_double), ("phi_deg", C.c_double)]


class rcwa_result_conical(C.Structure):
    _fields_ = [(name, C.c_void_p) for name in (
        "Jr", "Jt", "DEr", "DEt", "status", "eig_info", "n_eig", "n_dense_solve", "n_schur", "min_abs_lambda",
        "degenerate_mode_warning", "kx", "ky", "flux_r", "flux_t", "n_lu")]


class rcwa_gpu_config(C.Structure):
    _fields_ = [("device", C.c_int), ("workspace_limit", C.c_size_t)]


def cplx(z):
    z = complex(z)
    return rcwa_complex(z.real, z.imag)


def marshal_stack1d(stack):
    """Build an rcwa_stack1d from an object with nI, nII, period and layers (each layer with d,
    homogeneous, n, edges, n_values). Returns (struct, keepalive)."""
    keep = []
    layers = (rcwa_layer1d * max(1, len(stack.layers)))()
    for k, L in enumerate(stack.layers):
        s = layers[k]
        s.d = float(L.d)
        s.homogeneous = 1 if L.homogeneous else 0
        s.n = cplx(L.n if L.homogeneous else 1.0)
        s.fourier_method = int(getattr(L, "fourier_method", 0))
        s.fft_samples = int(getattr(L, "fft_samples", 0))
        if not L.homogeneous:
            e = np.ascontiguousarray(np.asarray(L.edges, dtype=np.float64))
            v = np.ascontiguousarray(np.asarray(L.n_values, dtype=np.complex128))
            keep += [e, v]
            s.n_segments = len(v)
            s.edges = e.ctypes.data_as(C.POINTER(C.c_double))
            s.n_values = C.cast(v.ctypes.data, C.POINTER(rcwa_complex))
        else:
            s.n_segments = 0
    st = rcwa_stack1d()
    st.nI = cplx(stack.nI)
    st.nII = cplx(stack.nII)
    st.period = float(stack.period)
    st.n_layers = len(stack.layers)
    st.layers = C.cast(layers, C.POINTER(rcwa_layer1d))
    keep.append(layers)
    return st, keep


def points_array(points):
    """Sweep points as an (n, 2) float64 array of (wavelength, theta_deg)."""
    p = np.ascontiguousarray(np.asarray(points, dtype=np.float64).reshape(-1, 2))
    return p


def result_views(n_points, M, with_diag=True):
    """Host arrays for rcwa_result1d and the struct pointing at them."""
    n = 2 * M + 1
    arrays = {
        "R": np.empty((n_points, n), np.complex128),
        "T": np.empty((n_points, n), np.complex128),
        "DEr": np.empty((n_points, n), np.float64),
        "DEt": np.empty((n_points, n), np.float64),
        "status": np.empty(n_points, np.int32),
        "eig_info": np.empty(n_points, np.int32),
        "n_eig": np.empty(n_points, np.int32),
        "n_dense_solve": np.empty(n_points, np.int32),
        "max_eig_residual": np.zeros(n_points, np.float64),
        "n_lu": np.empty(n_points, np.int32),
    }
    res = rcwa_result1d()
    for name, arr in arrays.items():
        setattr(res, name, arr.ctypes.data)
    return res, arrays


def conical_views(n_points, M):
    """Host arrays for rcwa_result_conical and the struct pointing at them."""
    n = 2 * M + 1
    arrays = {
        "Jr": np.empty((n_points, n, 4), np.complex128),
        "Jt": np.empty((n_points, n, 4), np.complex128),
        "DEr": np.empty((n_points, n, 4), np.float64),
        "DEt": np.empty((n_points, n, 4), np.float64),
        "status": np.empty(n_points, np.int32),
        "eig_info": np.empty(n_points, np.int32),
        "n_eig": np.empty(n_points, np.int32),
        "n_dense_solve": np.empty(n_points, np.int32),
        "n_schur": np.empty(n_points, np.int32),
        "min_abs_lambda": np.empty(n_points, np.float64),
        "degenerate_mode_warning": np.empty(n_points, np.int32),
        "kx": np.empty((n_points, n), np.float64),
        "ky": np.empty(n_points, np.float64),
        "flux_r": np.empty((n_points, n), np.float64),
        "flux_t": np.empty((n_points, n), np.float64),
        "n_lu": np.empty(n_points, np.int32),
    }
    res = rcwa_result_conical()
    for name, arr in arrays.items():
        setattr(res, name, arr.ctypes.data)
    return res, arrays


def conical_points_array(points):
    return np.ascontiguousarray(np.asarray(points, dtype=np.float64).reshape(-1, 3))


# ---------------------------------------------------------------- 2-D crossed gratings

RCWA_SAMPLE_RAYLEIGH = 3
RCWA_FACTORIZATION_LI = 0
RCWA_FACTORIZATION_LAURENT = 1


class rcwa_xprofile2d(C.Structure):
    _fields_ = [("n_segments", C.c_int), ("edges", C.POINTER(C.c_double)), ("n_values", C.POINTER(rcwa_complex))]


class rcwa_layer2d(C.Structure):
    _fields_ = [
        ("d", C.c_double),
        ("homogeneous", C.c_int),
        ("n", rcwa_complex),
        ("n_strips", C.c_int),
        ("y_edges", C.POINTER(C.c_double)),
        ("x_profiles", C.POINTER(rcwa_xprofile2d)),
    ]


class rcwa_stack2d(C.Structure):
    _fields_ = [
        ("nI", C.c_double),
        ("nII", rcwa_complex),
        ("Lx", C.c_double),
        ("Ly", C.c_double),
        ("n_layers", C.c_int),
        ("layers", C.POINTER(rcwa_layer2d)),
    ]


class rcwa_point2d(C.Structure):
    _fields_ = [("wavelength", C.c_double), ("theta_deg", C.c_double), ("phi_deg", C.c_double),
                ("Es", rcwa_complex), ("Ep", rcwa_complex)]


RESULT2D_FIELDS = ("Kx", "Ky", "kzI", "kzII", "Ex_r", "Ey_r", "Ez_r", "Ex_t", "Ey_t", "Ez_t", "Rs", "Rp", "Ts", "Tp",
                   "DEr", "DEt", "prop_r", "prop_t", "status", "eig_info", "n_eig", "n_dense_solve",
                   "max_eig_residual", "rayleigh_regions")


class rcwa_result2d(C.Structure):
    _fields_ = [(name, C.c_void_p) for name in RESULT2D_FIELDS]


def marshal_layer2d(L, s, keep):
    """Fill the rcwa_layer2d s from a Layer2D-like object; arrays it points at are appended to keep."""
    s.d = float(L.d)
    s.homogeneous = 1 if L.homogeneous else 0
    s.n = cplx(L.n if L.homogeneous else 1.0)
    if L.homogeneous:
        s.n_strips = 0
        return
    ye = np.ascontiguousarray(np.asarray(L.y_edges, dtype=np.float64))
    rows = (rcwa_xprofile2d * max(1, len(L.x_profiles)))()
    keep += [ye, rows]
    for k, p in enumerate(L.x_profiles):
        e = np.ascontiguousarray(np.asarray(p.edges, dtype=np.float64))
        v = np.ascontiguousarray(np.asarray(p.n_values, dtype=np.complex128))
        keep += [e, v]
        rows[k].n_segments = len(v)
        rows[k].edges = e.ctypes.data_as(C.POINTER(C.c_double))
        rows[k].n_values = C.cast(v.ctypes.data, C.POINTER(rcwa_complex))
    s.n_strips = len(L.x_profiles)
    s.y_edges = ye.ctypes.data_as(C.POINTER(C.c_double))
    s.x_profiles = C.cast(rows, C.POINTER(rcwa_xprofile2d))


def marshal_stack2d(stack):
    """rcwa_stack2d from a Stack2D-like object. Returns (struct, keepalive)."""
    keep = []
    layers = (rcwa_layer2d * max(1, len(stack.layers)))()
    for k, L in enumerate(stack.layers):
        marshal_layer2d(L, layers[k], keep)
    st = rcwa_stack2d()
    st.nI = float(stack.nI)
    st.nII = cplx(stack.nII)
    st.Lx = float(stack.Lx)
    st.Ly = float(stack.Ly)
    st.n_layers = len(stack.layers)
    st.layers = C.cast(layers, C.POINTER(rcwa_layer2d))
    keep.append(layers)
    return st, keep


def points2d_array(points):
    """Points (wavelength, theta_deg, phi_deg, Es, Ep) as an rcwa_point2d array."""
    pts = (rcwa_point2d * max(1, len(points)))()
    for k, (wl, th, ph, es, ep) in enumerate(points):
        pts[k].wavelength = float(wl)
        pts[k].theta_deg = float(th)
        pts[k].phi_deg = float(ph)
        pts[k].Es = cplx(es)
        pts[k].Ep = cplx(ep)
    return pts


def result2d_views(n_points, N, n_layers):
    """Host arrays for rcwa_result2d and the struct pointing at them."""
    arrays = {}
    for name in ("Kx", "Ky", "DEr", "DEt"):
        arrays[name] = np.empty((n_points, N), np.float64)
    for name in ("kzI", "kzII", "Ex_r", "Ey_r", "Ez_r", "Ex_t", "Ey_t", "Ez_t", "Rs", "Rp", "Ts", "Tp"):
        arrays[name] = np.empty((n_points, N), np.complex128)
    arrays["prop_r"] = np.empty((n_points, N), np.uint8)
    arrays["prop_t"] = np.empty((n_points, N), np.uint8)
    for name in ("status", "eig_info", "n_eig", "n_dense_solve"):
        arrays[name] = np.empty(n_points, np.int32)
    arrays["max_eig_residual"] = np.zeros(n_points, np.float64)
    arrays["rayleigh_regions"] = np.zeros((n_points, n_layers + 2), np.uint8)
    res = rcwa_result2d()
    for name, arr in arrays.items():
        setattr(res, name, arr.ctypes.data)
    return res, arrays


# ---------------------------------------------------------------- serving

RCWA_ETIMEOUT = -6
RCWA_ENUMERIC = -7
RCWA_ECANCELLED = -8
RCWA_SLICE_XZ, RCWA_SLICE_YZ = 0, 1
RCWA_PHASE_ABSOLUTE, RCWA_PHASE_INCIDENT, RCWA_PHASE_CUSTOM = 0, 1, 2
RCWA_UNWRAP_NONE, RCWA_UNWRAP_X, RCWA_UNWRAP_Z, RCWA_UNWRAP_BOTH = 0, 1, 2, 3
RCWA_REQ_1D = 0
RCWA_REQ_CONICAL = 1
RCWA_REQ_2D = 2


class rcwa_server_config(C.Structure):
    _fields_ = [("device", C.c_int), ("slots", C.c_int), ("hbm_budget", C.c_size_t), ("max_bypass_ms", C.c_int),
                ("max_batch", C.c_int)]


class rcwa_request(C.Structure):
    _fields_ = [
        ("kind", C.c_int),
        ("stack1d", C.POINTER(rcwa_stack1d)),
        ("stack2d", C.POINTER(rcwa_stack2d)),
        ("wavelength", C.c_double),
        ("theta_deg", C.c_double),
        ("phi_deg", C.c_double),
        ("M", C.c_int),
        ("polarization", C.c_int),
        ("M1", C.c_int),
        ("M2", C.c_int),
        ("factorization", C.c_int),
        ("Es", rcwa_complex),
        ("Ep", rcwa_complex),
        ("options", rcwa_options),
    ]


class rcwa_response(C.Structure):
    _fields_ = [("code", C.c_int), ("slot", C.c_int), ("submit_s", C.c_double), ("start_s", C.c_double),
                ("finish_s", C.c_double), ("footprint_bytes", C.c_double), ("batch", C.c_int)]
