"""ctypes binding of the CPU oracle (oracle/fpde_oracle.c).

Test infrastructure: imported only by tests/, the smoke check and the CPU-baseline leg
of bench.py, to check results. The GPU library never loads it. ``load()`` builds the
shared object with ``make -C oracle`` on first use (a second or two with gcc).
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(HERE, "_build", "libfpde_oracle.so")
_lib = None

_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")


def build():
    subprocess.check_call(["make", "-s", "-C", HERE], stdout=subprocess.DEVNULL)
    return _LIB_PATH


def load():
    global _lib
    if _lib is not None:
        return _lib
    src = os.path.join(HERE, "fpde_oracle.c")
    if (not os.path.exists(_LIB_PATH)) or os.path.getmtime(_LIB_PATH) < os.path.getmtime(src):
        build()
    lib = C.CDLL(_LIB_PATH)
    i64, i32, d = C.c_int64, C.c_int, C.c_double
    vp = C.c_void_p
    lib.fo_l1_weights.argtypes = [d, _dp, i32, _dp, C.POINTER(d)]
    lib.fo_l1_sum.argtypes = [_dp, i64, i32, _dp, _dp, i64, i64, _dp]
    lib.fo_l1_sum_snapshots.argtypes = [_dp, i64, i32, _dp, _dp, i64, _dp]
    lib.fo_weights_g.argtypes = [d, d, _dp, i32, _dp, C.POINTER(d)]
    lib.fo_sum_restricted.argtypes = [_dp, i64, i32, _dp, _dp, d, i32, i64, _dp]
    lib.fo_sum_series.argtypes = [_dp, _dp, i64, _dp, i32, _dp, d, d, d, d, _dp]
    lib.fo_thomas_line.argtypes = [i32, _dp, _dp, _dp, _dp, i32, d, i32, d, d, _dp]
    lib.fo_line_coefs.argtypes = [i32, _dp, _dp, _dp, _dp, _dp, _dp]
    lib.fo_line_step.argtypes = [i32, _dp, _dp, i64, i32, _dp, _dp, d, d, _dp, _dp, _dp, vp,
                                 i32, d, i32, d, d, vp]
    lib.fo_line_step.restype = i32
    lib.fo_line_run.argtypes = [i32, _dp, _dp, i64, i32, d, d, d, _dp, _dp, _dp, i32, d, i32, d, d]
    lib.fo_line_run.restype = i32
    lib.fo_line_run_general.argtypes = [i32, _dp, _dp, i64, i32, _dp, d, _dp, _dp, _dp, vp, i32, i32, d, i32, d, d]
    lib.fo_line_run_general.restype = i32
    lib.fo_lod_step_dirichlet.argtypes = [i32, i32, i32, _dp, _dp, i32, _dp, _dp, d, d,
                                          _dp, _dp, _dp, _dp, _dp, vp]
    lib.fo_lod_step_dirichlet.restype = i32
    lib.fo_lod_step.argtypes = [i32, i32, i32, _dp, _dp, i32, _dp, _dp, d, d, _dp, _dp, _dp, vp, _dp,
                                _ip, _ip, _dp, vp]
    lib.fo_lod_step.restype = i32
    lib.fo_lod_step_dirichlet_sum.argtypes = [i32, i32, i32, _dp, _dp, i32, _dp, d, d, _dp, _dp, _dp, _dp, _dp,
                                              _dp]
    lib.fo_lod_step_dirichlet_sum.restype = i32
    lib.fo_richards_closures.argtypes = [i32, _dp, i32, d, vp, vp, vp]
    lib.fo_lod_step_richards.argtypes = [i32, i32, i32, _dp, _dp, i32, _dp, _dp, d, d, _dp, _dp, _dp, _dp, i32, d,
                                         d, vp, vp]
    lib.fo_lod_step_richards.restype = i32
    lib.fo_lod_step_richards_salt.argtypes = [i32, i32, i32, _dp, _dp, i32, _dp, _dp, d, d, _dp, _dp, _dp, _dp, i32,
                                              d, d, vp, vp, vp, vp, vp, vp, vp, d, d, vp]
    lib.fo_lod_step_richards_salt.restype = i32
    lib.fo_line_run_richards.argtypes = [i32, _dp, _dp, i64, i32, d, d, d, _dp, _dp, i32, d, _dp, i32, vp, i32,
                                         i32, d, d]
    lib.fo_line_run_richards.restype = i32
    lib.fo_sf_matvec.argtypes = [i32, _dp, _dp, _dp, vp, vp, i32, _dp, _dp, _dp]
    lib.fo_sf_solve.argtypes = [i32, _dp, _dp, _dp, vp, vp, i32, _dp, _dp, d, i32]
    lib.fo_sf_solve.restype = i32
    lib.fo_lod_step_sf.argtypes = [i32, i32, i32, _dp, _dp, i32, _dp, _dp, d, d, _dp, _dp, _dp, _dp, _dp, _dp, i32,
                                   i32, d, i32, vp, _dp, vp, C.POINTER(i64), vp, vp]
    lib.fo_lod_step_sf.restype = i32
    lib.fo_sf3d_matvec.argtypes = [i32, i32, i32, _dp, _dp, C.POINTER(C.c_void_p), vp, vp, i32, _dp, _dp, _dp]
    lib.fo_sf3d_solve.argtypes = [i32, i32, i32, _dp, _dp, C.POINTER(C.c_void_p), vp, vp, i32, _dp, _dp, d, i32]
    lib.fo_sf3d_solve.restype = i32
    lib.fo_lod_step_sf3d.argtypes = [i32, i32, i32, _dp, C.POINTER(d), _dp, i32, _dp, _dp, d, d, _dp, _dp, _dp,
                                     _dp, _dp, _dp, i32, i32, d, i32, vp, _dp, vp, vp, vp, C.POINTER(i64), vp, vp]
    lib.fo_caputo_derivative.argtypes = [i32, d, d, d, _dp, _dp]
    lib.fo_do_derivative.argtypes = [i32, d, i32, _dp, _dp, _dp, i32, i32, i32, _dp]
    lib.fo_do_fused_weights.argtypes = [i32, _dp, _dp, _dp, d, i32, _dp]
    lib.fo_do_eq_solve.argtypes = [i32, i32, i32, i32, i32, d, d, d, _dp, _dp, _dp, C.POINTER(d)]
    lib.fo_do_eq_solve.restype = i32
    _lib = lib
    return lib


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def time_points(taus):
    """Time[0] = 0, Time[k+1] = Time[k] + tau[k] (the reference accumulates the same way)."""
    t = np.zeros(len(taus) + 1)
    for k, v in enumerate(taus):
        t[k + 1] = t[k] + v
    return t


def l1_weights(alpha, time, n):
    lib = load()
    kb = np.zeros(max(n, 1))
    k0 = C.c_double()
    lib.fo_l1_weights(alpha, np.ascontiguousarray(time, dtype=np.float64), n, kb, C.byref(k0))
    return kb[:n], k0.value


def l1_sum(D, n, kb, tau, i0=0, i1=None):
    lib = load()
    D = np.ascontiguousarray(D, dtype=np.float64)
    P = D.shape[-1]
    i1 = P if i1 is None else i1
    S = np.zeros(P)
    lib.fo_l1_sum(D.reshape(-1), P, n, np.ascontiguousarray(kb, dtype=np.float64),
                  np.ascontiguousarray(tau, dtype=np.float64), i0, i1, S)
    return S


def l1_sum_snapshots(old, kb, tau):
    lib = load()
    old = np.ascontiguousarray(old, dtype=np.float64)
    nold, OS = old.shape
    S = np.zeros(OS)
    lib.fo_l1_sum_snapshots(old.reshape(-1), OS, nold, np.ascontiguousarray(kb, dtype=np.float64),
                            np.ascontiguousarray(tau, dtype=np.float64), OS, S)
    return S


def weights_g(p, alpha, time, n):
    """kb (n values) and kkk0 of step n for g(t) = t^p (fo_weights_g)."""
    lib = load()
    kb = np.zeros(max(n, 1))
    k0 = C.c_double()
    lib.fo_weights_g(p, alpha, np.ascontiguousarray(time, dtype=np.float64), n, kb, C.byref(k0))
    return kb[:n], k0.value


def sum_restricted(old, kb, tau, thr, bs=0):
    lib = load()
    old = np.ascontiguousarray(old, dtype=np.float64)
    nold, OS = old.shape
    S = np.zeros(OS)
    lib.fo_sum_restricted(old.reshape(-1), OS, nold, np.ascontiguousarray(kb, dtype=np.float64),
                          np.ascontiguousarray(tau, dtype=np.float64), thr, bs, OS, S)
    return S


def sum_series(prev, cur, H, row2, gt, gtj, alpha, tau_t):
    """One step of the series-expansion history; H (nodes, P) is updated in place."""
    lib = load()
    assert H.dtype == np.float64 and H.flags["C_CONTIGUOUS"]
    nodes, P = H.shape
    S = np.zeros(nodes)
    lib.fo_sum_series(np.ascontiguousarray(prev, dtype=np.float64), np.ascontiguousarray(cur, dtype=np.float64),
                      nodes, H.reshape(-1), P, np.ascontiguousarray(row2, dtype=np.float64), gt, gtj, alpha,
                      tau_t, S)
    return S


def thomas_line(A, B, R, Om, ltype, g0, rtype, gN, dLN, U):
    lib = load()
    U = np.array(U, dtype=np.float64)
    N = len(U) - 1
    lib.fo_thomas_line(N, *(np.ascontiguousarray(x, dtype=np.float64) for x in (A, B, R, Om)),
                       ltype, g0, rtype, gN, dLN, U)
    return U


def line_coefs(k, iw, dL):
    lib = load()
    N = len(k) - 1
    A, B, Rl = np.zeros(N + 1), np.zeros(N + 1), np.zeros(N + 1)
    lib.fo_line_coefs(N, *(np.ascontiguousarray(x, dtype=np.float64) for x in (k, iw, dL)), A, B, Rl)
    return A, B, Rl


def line_run(U0, steps, tau, alpha, Da, A, B, Rl, ltype=0, g0=0.0, rtype=0, gN=0.0, dLN=0.0,
             P=None):
    """Full run of the 1D line problem; returns the final state and the increment history."""
    lib = load()
    U = np.array(U0, dtype=np.float64)
    N = len(U) - 1
    P = P or (N + 1)
    hist = np.zeros((steps, P))
    lib.fo_line_run(N, U, hist.reshape(-1), P, steps, tau, alpha, Da,
                    *(np.ascontiguousarray(x, dtype=np.float64) for x in (A, B, Rl)),
                    ltype, g0, rtype, gN, dLN)
    return U, hist


def line_run_general(U0, steps, w, theta, A, B, Rl, src=None, ltype=0, g0=0.0, rtype=0, gN=0.0, dLN=0.0):
    """Line run with explicit lag weights w (w[0] local), explicit fraction theta and an
    optional source (rows x (N+1); step n uses row min(n, rows-1)). Returns (U, hist)."""
    lib = load()
    U = np.array(U0, dtype=np.float64)
    N = len(U) - 1
    hist = np.zeros((steps, N + 1))
    w = np.ascontiguousarray(w, dtype=np.float64)
    assert len(w) >= steps + 1
    rows = 0
    sp = None
    if src is not None:
        src = np.ascontiguousarray(np.atleast_2d(src), dtype=np.float64)
        assert src.shape[1] == N + 1
        rows = src.shape[0]
        sp = src.ctypes.data_as(C.c_void_p)
    lib.fo_line_run_general(N, U, hist.reshape(-1), N + 1, steps, w, theta,
                            *(np.ascontiguousarray(x, dtype=np.float64) for x in (A, B, Rl)),
                            sp, rows, ltype, g0, rtype, gN, dLN)
    return U, hist


def lod_step_dirichlet(dims, U, hist, n, kb, tau, Da, kkk0, coefA, coefB, coefRlap, rp, bc, want_S=False):
    lib = load()
    sN, M, K = dims
    S = np.zeros_like(U) if want_S else None
    lib.fo_lod_step_dirichlet(sN, M, K, U.reshape(-1), hist.reshape(-1), n,
                              np.ascontiguousarray(kb, dtype=np.float64),
                              np.ascontiguousarray(tau, dtype=np.float64), Da, kkk0,
                              coefA.reshape(-1), coefB.reshape(-1), coefRlap.reshape(-1),
                              rp.reshape(-1), bc.reshape(-1), _ptr(S))
    return S



def lod_step_dirichlet_sum(dims, U, hist, n, tau, Da, kkk0, coefA, coefB, coefRlap, rp, bc, S):
    """The Dirichlet step with the history sums S (grid) given: the reference's sum_alg 2 runs."""
    lib = load()
    sN, M, K = dims
    lib.fo_lod_step_dirichlet_sum(sN, M, K, U.reshape(-1), hist.reshape(-1), n,
                                  np.ascontiguousarray(tau, dtype=np.float64), Da, kkk0,
                                  coefA.reshape(-1), coefB.reshape(-1), coefRlap.reshape(-1),
                                  rp.reshape(-1), bc.reshape(-1),
                                  np.ascontiguousarray(S, dtype=np.float64).reshape(-1))


def lod_step(dims, U, hist, n, kb, tau, Da, kkk0, coefA, coefB, coefRlap, rp, bc, lkind=(0, 0, 0),
             rkind=(0, 0, 0), dLN=(0.0, 0.0, 0.0), want_S=False):
    """fo_lod_step: one LOD step with boundary kinds per pass (0 sN, 1 _M, 2 K); rp may be None."""
    lib = load()
    sN, M, K = dims
    S = np.zeros_like(U) if want_S else None
    rpp = None if rp is None else np.ascontiguousarray(rp, dtype=np.float64).reshape(-1)
    lib.fo_lod_step(sN, M, K, U.reshape(-1), hist.reshape(-1), n,
                    np.ascontiguousarray(kb, dtype=np.float64), np.ascontiguousarray(tau, dtype=np.float64),
                    Da, kkk0, coefA.reshape(-1), coefB.reshape(-1), coefRlap.reshape(-1),
                    None if rpp is None else rpp.ctypes.data_as(C.c_void_p),
                    np.ascontiguousarray(bc, dtype=np.float64).reshape(-1),
                    np.array(lkind, dtype=np.int32), np.array(rkind, dtype=np.int32),
                    np.array(dLN, dtype=np.float64), _ptr(S))
    return S


def lod_run(dims, U0, steps, tau, alpha, Da, coefA, coefB, coefRlap, rp=None, bc=None, lkind=(0, 0, 0),
            rkind=(0, 0, 0), dLN=(0.0, 0.0, 0.0)):
    """Uniform-tau LOD run with the closed-form weights; returns the final grid."""
    sN, M, K = dims
    U = np.array(U0, dtype=np.float64)
    G = U.shape
    hist = np.zeros((steps,) + G)
    taus = np.full(steps + 1, tau)
    time = time_points(taus)
    bc = np.zeros(G) if bc is None else bc
    for n in range(steps):
        kb, k0 = l1_weights(alpha, time, n)
        lod_step(dims, U, hist, n, kb if n else np.zeros(1), taus, Da, k0, coefA, coefB, coefRlap, rp, bc,
                 lkind, rkind, dLN)
    return U


def richards_closures(P, kform, ksat):
    """(wetness, inv_dw_dh, KK) of the reference's Richards problem at suctions P (metres)."""
    lib = load()
    P = np.ascontiguousarray(P, dtype=np.float64)
    w, iw, kk = np.zeros_like(P), np.zeros_like(P), np.zeros_like(P)
    lib.fo_richards_closures(len(P), P, kform, ksat, _ptr(w), _ptr(iw), _ptr(kk))
    return w, iw, kk


def lod_step_richards(dims, U, hist, n, kb, tau, Da, kkk0, sZ, sdL, dLx, dLy, kform, ksat, E, rp=None,
                      want_S=False):
    """fo_lod_step_richards: one LOD step of the Richards problem (coefficients from the grid)."""
    lib = load()
    sN, M, K = dims
    S = np.zeros_like(U) if want_S else None
    f = lambda x: np.ascontiguousarray(x, dtype=np.float64)
    rpp = None if rp is None else f(rp).reshape(-1)
    lib.fo_lod_step_richards(sN, M, K, U.reshape(-1), hist.reshape(-1), n, f(kb), f(tau), Da, kkk0, f(sZ), f(sdL),
                             f(dLx), f(dLy), kform, ksat, E,
                             None if rpp is None else rpp.ctypes.data_as(C.c_void_p), _ptr(S))
    return S


def lod_step_richards_salt(dims, U, hist, n, kb, tau, Da, kkk0, sZ, sdL, dLx, dLy, kform, ksat, E, C, histC, cA, cB,
                           cR, nu, sigma, rp=None, want_S=False):
    """fo_lod_step_richards_salt: one LOD step of H and the salt concentration C (equation 1),
    both advanced in place; cA/cB/cR: equation 1's coefficient grids (3 passes). Returns
    (S_H, S_C) when want_S."""
    lib = load()
    sN, M, K = dims
    S = np.zeros_like(U) if want_S else None
    SC = np.zeros_like(U) if want_S else None
    rpp = None if rp is None else _f64(rp).reshape(-1)
    lib.fo_lod_step_richards_salt(sN, M, K, U.reshape(-1), hist.reshape(-1), n, _f64(kb), _f64(tau), Da, kkk0,
                                  _f64(sZ), _f64(sdL), _f64(dLx), _f64(dLy), kform, ksat, E, _ptr(rpp), _ptr(S),
                                  _ptr(C), _ptr(histC), _ptr(_f64(cA)), _ptr(_f64(cB)), _ptr(_f64(cR)), nu, sigma,
                                  _ptr(SC))
    return (S, SC) if want_S else None


def line_run_richards(U0, steps, tau, alpha, Da, Z, dL, kform, ksat, E, src=None, rtype=0, gN=0.0, dLN=0.0):
    """fo_line_run_richards: a Richards line with the history. Returns (U, hist)."""
    lib = load()
    U = np.array(U0, dtype=np.float64)
    N = len(U) - 1
    hist = np.zeros((steps, N + 1))
    f = lambda x: np.ascontiguousarray(x, dtype=np.float64)
    E = np.atleast_1d(f(E))
    rows, sp = 0, None
    if src is not None:
        src = f(np.atleast_2d(src))
        rows, sp = src.shape[0], src.ctypes.data_as(C.c_void_p)
    lib.fo_line_run_richards(N, U, hist.reshape(-1), N + 1, steps, tau, alpha, Da, f(Z), f(dL), kform, ksat, E, len(E),
                             sp, rows, rtype, gN, dLN)
    return U, hist


def _f64(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.float64)


def sf_matvec(mat, mc, Tm, x, iw=None, rs=None, space_der=0):
    """fo_sf_matvec (vmul_T, toeplitz_mult_alg 0) on one line: mat, mc are 3 x (n+1)."""
    lib = load()
    x = _f64(x)
    n = x.size - 1
    r = np.zeros(n + 1)
    bt = np.zeros(n + 1)
    iw, rs = _f64(iw), _f64(rs)
    lib.fo_sf_matvec(n, _f64(mat).reshape(-1), _f64(mc).reshape(-1), _f64(Tm), _ptr(iw), _ptr(rs), space_der, x,
                     r, bt)
    return r


def sf_solve(mat, mc, Tm, B, x0, thr, maxiter, iw=None, rs=None, space_der=0):
    """fo_sf_solve (solve_mln<1> with vmul_T): returns (solution, iterations)."""
    lib = load()
    x = _f64(x0).copy()
    n = x.size - 1
    iw, rs = _f64(iw), _f64(rs)
    it = lib.fo_sf_solve(n, _f64(mat).reshape(-1), _f64(mc).reshape(-1), _f64(Tm), _ptr(iw), _ptr(rs), space_der,
                         _f64(B), x, thr, maxiter)
    return x, it


def _ends(rkind, dLN):
    """The far-end kinds (3 ints) and steps (3 doubles) of the passes as C arrays, or (None, None)."""
    if rkind is None:
        return None, None, None
    rk = np.ascontiguousarray(rkind, dtype=np.int32)
    dl = np.ascontiguousarray(dLN, dtype=np.float64)
    return rk.ctypes.data_as(C.c_void_p), dl.ctypes.data_as(C.c_void_p), (rk, dl)


def lod_step_sf(dims, U, hist, n, kb, tau, Da, kkk0, coefA, coefB, coefRlap, mc, iw, Tm, space_der, thr, maxiter,
                rp, bc, want_S=False, rkind=None, dLN=None):
    """fo_lod_step_sf: one LOD step with the implicit space-fractional line solves.
    mc: (3 passes, 3, G), iw: (3, G), Tm: (3, ldt); rkind/dLN: far-end kinds and steps per pass
    (1 = the flux row of bottom_cond 0). Returns (S or None, iterations)."""
    lib = load()
    sN, M, K = dims
    S = np.zeros_like(U) if want_S else None
    Tm = _f64(Tm)
    it = C.c_int64()
    rpp = None if rp is None else _f64(rp).reshape(-1)
    ends = _ends(rkind, dLN)                   # keeps the arrays alive through the call
    lib.fo_lod_step_sf(sN, M, K, U.reshape(-1), hist.reshape(-1), n, _f64(kb), _f64(tau), Da, kkk0,
                       _f64(coefA).reshape(-1), _f64(coefB).reshape(-1), _f64(coefRlap).reshape(-1),
                       _f64(mc).reshape(-1), _f64(iw).reshape(-1), Tm.reshape(-1), Tm.shape[1], space_der, thr,
                       maxiter, _ptr(rpp), _f64(bc).reshape(-1), _ptr(S), C.byref(it), *ends[:2])
    return S, it.value


def _rows3(Tm):
    """Three Toeplitz rows (one per axis: sN, _M, K) as a C array of pointers; keeps the arrays alive."""
    rows = [_f64(t) for t in Tm]
    arr = (C.c_void_p * 3)(*[r.ctypes.data_as(C.c_void_p).value for r in rows])
    return arr, rows


def sf3d_matvec(dims, mat, mc, Tm, x, iw=None, rs=None, space_der=0):
    """fo_sf3d_matvec (vmul_T_3d): mat 7 x V, mc 9 x V, Tm three rows, iw 3 x V, V = G + 1."""
    lib = load()
    sN, M, K = dims
    x = _f64(x).reshape(-1)
    r = np.zeros_like(x)
    bt = np.zeros_like(x)
    arr, keep = _rows3(Tm)
    iw, rs = _f64(iw), _f64(rs)
    lib.fo_sf3d_matvec(sN, M, K, _f64(mat).reshape(-1), _f64(mc).reshape(-1), arr,
                       _ptr(None if iw is None else iw.reshape(-1)), _ptr(rs), space_der, x, r, bt)
    return r


def sf3d_solve(dims, mat, mc, Tm, B, x0, thr, maxiter, iw=None, rs=None, space_der=0):
    """fo_sf3d_solve (solve_mln<1> with vmul_T_3d): returns (solution, iterations)."""
    lib = load()
    sN, M, K = dims
    x = _f64(x0).reshape(-1).copy()
    arr, keep = _rows3(Tm)
    iw, rs = _f64(iw), _f64(rs)
    it = lib.fo_sf3d_solve(sN, M, K, _f64(mat).reshape(-1), _f64(mc).reshape(-1), arr,
                           _ptr(None if iw is None else iw.reshape(-1)), _ptr(rs), space_der,
                           _f64(B).reshape(-1), x, thr, maxiter)
    return x, it


def lod_step_sf3d(dims, U, u_end, hist, n, kb, tau, Da, kkk0, coefA, coefB, coefRlap, mc, iw, Tm, space_der, thr,
                  maxiter, rp, bc, want_system=False, rkind=None, dLN=None):
    """fo_lod_step_sf3d: one step of the fully implicit 3D scheme. U (G values) is advanced in place.
    Returns (u_end, iterations, mat 7 x V or None, Om or None, S or None)."""
    lib = load()
    sN, M, K = dims
    G = U.size
    V = G + 1
    Tm = _f64(Tm)
    it = C.c_int64()
    ue = C.c_double(u_end)
    mat = np.zeros((7, V)) if want_system else None
    om = np.zeros(V) if want_system else None
    S = np.zeros(G) if want_system else None
    rpp = None if rp is None else _f64(rp).reshape(-1)
    ends = _ends(rkind, dLN)
    lib.fo_lod_step_sf3d(sN, M, K, U.reshape(-1), C.byref(ue), hist.reshape(-1), n, _f64(kb), _f64(tau), Da, kkk0,
                         _f64(coefA).reshape(-1), _f64(coefB).reshape(-1), _f64(coefRlap).reshape(-1),
                         _f64(mc).reshape(-1), _f64(iw).reshape(-1), Tm.reshape(-1), Tm.shape[1], space_der, thr,
                         maxiter, _ptr(rpp), _f64(bc).reshape(-1), _ptr(mat), _ptr(om), _ptr(S), C.byref(it),
                         *ends[:2])
    return ue.value, it.value, mat, om, S


def caputo_derivative(F, tau, a, g2a):
    lib = load()
    F = np.ascontiguousarray(F, dtype=np.float64)
    DF = np.zeros(len(F))
    lib.fo_caputo_derivative(len(F), tau, a, g2a, F, DF)
    return DF


def do_derivative(F, tau, WA, gs, maxt=-1, t0=1, j0=0):
    lib = load()
    F = np.ascontiguousarray(F, dtype=np.float64)
    DF = np.zeros(len(F))
    lib.fo_do_derivative(len(F), tau, len(WA), np.ascontiguousarray(WA, dtype=np.float64),
                         np.ascontiguousarray(gs, dtype=np.float64), F, maxt, t0, j0, DF)
    return DF


def do_fused_weights(aq, Wq, gq, tau, nl):
    lib = load()
    c = np.zeros(nl)
    lib.fo_do_fused_weights(len(aq), *(np.ascontiguousarray(x, dtype=np.float64) for x in (aq, Wq, gq)),
                            tau, nl, c)
    return c


def do_eq_solve(ex, C0, Nt, tblock, h, tau, D, WA, gs):
    lib = load()
    Nx = len(C0)
    Cm = np.zeros((Nx, Nt))
    Cm[:, 0] = C0
    b0 = C.c_double()
    lib.fo_do_eq_solve(ex, Nx, Nt, tblock, len(WA), h, tau, D,
                       np.ascontiguousarray(WA, dtype=np.float64),
                       np.ascontiguousarray(gs, dtype=np.float64), Cm.reshape(-1), C.byref(b0))
    return Cm, b0.value
