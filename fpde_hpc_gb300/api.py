"""Pythonic wrappers over the C ABI (host numpy arrays or CUDA torch tensors)."""
import ctypes as C

import numpy as np

from ._lib import ColumnDesc, LineDesc, LineTuning, Lod3dDesc, Richards, Sf3dSystem, SpaceFrac, check, load

FP64, SPLIT_BF16, SPLIT_F16 = 0, 1, 2


def _is_dev(x):
    return hasattr(x, "is_cuda") and x.is_cuda


def _ptr(x):
    if x is None:
        return None
    if hasattr(x, "data_ptr"):
        if x.dtype.__str__() != "torch.float64" or not x.is_contiguous():
            raise TypeError("device buffers must be contiguous float64 tensors")
        return C.c_void_p(x.data_ptr())
    if not (isinstance(x, np.ndarray) and x.dtype == np.float64 and x.flags["C_CONTIGUOUS"]):
        raise TypeError("host buffers must be C-contiguous float64 numpy arrays")
    return x.ctypes.data_as(C.c_void_p)


def _f64(x):
    return x if _is_dev(x) else np.ascontiguousarray(x, dtype=np.float64)


def weights_l1(alpha, time, n):
    t = np.ascontiguousarray(time, dtype=np.float64)
    kb = np.zeros(max(n, 1))
    k0 = C.c_double()
    check(load().fpde_weights_l1(alpha, _ptr(t), n, _ptr(kb), C.byref(k0)), "fpde_weights_l1")
    return kb[:n], k0.value


def weights_l1_lags(alpha, n):
    b = np.zeros(max(n, 1))
    check(load().fpde_weights_l1_lags(alpha, n, _ptr(b)), "fpde_weights_l1_lags")
    return b[:n]


def gamma(x):
    out = C.c_double()
    check(load().fpde_gamma(x, C.byref(out)), "fpde_gamma")
    return out.value


def restricted_lags(kb_lag, eps):
    """Lags kept by restricted summing (fpde_restricted_lags): kb_lag[j] is the weight of lag j+1."""
    kb = np.ascontiguousarray(kb_lag, dtype=np.float64)
    out = C.c_int()
    check(load().fpde_restricted_lags(_ptr(kb) if kb.size else None, int(kb.size), float(eps), C.byref(out)),
          "fpde_restricted_lags")
    return out.value


def do_weights(orders, qw, tau, n, gnorm=None):
    """Fused distributed-order lag weights c[0..n-1] (fpde_do_weights)."""
    a = np.ascontiguousarray(orders, dtype=np.float64)
    q = np.ascontiguousarray(qw, dtype=np.float64)
    g = None if gnorm is None else np.ascontiguousarray(gnorm, dtype=np.float64)
    c = np.zeros(n)
    check(load().fpde_do_weights(len(a), _ptr(a), _ptr(q), None if g is None else _ptr(g), tau, n, _ptr(c)),
          "fpde_do_weights")
    return c


def autotune_line(ctx, N, alpha, tau, Da, A, B, Rlap, u0, max_steps, left=(0, 0.0), right=(0, 0.0), dLN=0.0,
                  precision=FP64, lag_weights=None, theta=0.0, source=None):
    """fpde_line_autotune: the fastest launch parameters for this line (a LineTuning to pass as
    Line(..., tuning=...))."""
    d = LineDesc(N=N, alpha=alpha, tau=tau, Da=Da, left_kind=left[0], left_value=left[1], right_kind=right[0],
                 right_value=right[1], dLN=dLN, precision=precision, max_steps=max_steps, theta=theta)
    keep = []
    if lag_weights is not None:
        w = np.ascontiguousarray(lag_weights, dtype=np.float64)
        keep.append(w)
        d.lag_weights = w.ctypes.data
    if source is not None:
        src = np.ascontiguousarray(np.atleast_2d(source), dtype=np.float64)
        keep.append(src)
        d.source, d.source_rows = src.ctypes.data, src.shape[0]
    arrs = [np.ascontiguousarray(x, dtype=np.float64) for x in (A, B, Rlap, u0)]
    out = LineTuning()
    check(ctx.lib.fpde_line_autotune(ctx.h, C.byref(d), *(_ptr(x) for x in arrs), C.byref(out)),
          "fpde_line_autotune")
    return out


def sf_toeplitz_row(gamma_, Z, n):
    """The Toeplitz row Tm[0..n] of a uniform axis with n+2 coordinates Z (fpde_sf_toeplitz_row)."""
    Z = np.ascontiguousarray(Z, dtype=np.float64)
    if Z.size < n + 2:
        raise ValueError("Z needs n+2 coordinates")
    Tm = np.zeros(n + 1)
    check(load().fpde_sf_toeplitz_row(float(gamma_), Z.ctypes.data_as(C.c_void_p), int(n),
                                      Tm.ctypes.data_as(C.c_void_p)), "fpde_sf_toeplitz_row")
    return Tm


def line_coefs(k, dL, iw=None):
    k = np.ascontiguousarray(k, dtype=np.float64)
    N = len(k) - 1
    dL = np.ascontiguousarray(dL, dtype=np.float64)
    A, B, R = np.zeros(N + 1), np.zeros(N + 1), np.zeros(N + 1)
    iwp = None if iw is None else _ptr(np.ascontiguousarray(iw, dtype=np.float64))
    check(load().fpde_line_coefs(N, _ptr(k), iwp, _ptr(dL), _ptr(A), _ptr(B), _ptr(R)), "fpde_line_coefs")
    return A, B, R


class Context:
    def __init__(self, device=0):
        self.lib = load()
        self.h = C.c_void_p()
        check(self.lib.fpde_ctx_create(device, C.byref(self.h)), "fpde_ctx_create")

    def close(self):
        if self.h:
            self.lib.fpde_ctx_destroy(self.h)
            self.h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def synchronize(self):
        check(self.lib.fpde_ctx_synchronize(self.h), "fpde_ctx_synchronize")

    def set_stream(self, stream_handle):
        check(self.lib.fpde_ctx_set_stream(self.h, C.c_void_p(stream_handle)), "fpde_ctx_set_stream")

    @property
    def sm_count(self):
        v = C.c_int()
        check(self.lib.fpde_ctx_sm_count(self.h, C.byref(v)), "fpde_ctx_sm_count")
        return v.value

    def sum_snapshots(self, old, kb, tau, nodes=None):
        """The reference Sum kernel contract: old is (old_size, OS) time-major snapshots."""
        dev = _is_dev(old)
        old = _f64(old)
        nold, OS = old.shape
        nodes = OS if nodes is None else nodes
        if dev:
            import torch
            S = torch.zeros(nodes, dtype=torch.float64, device=old.device)
        else:
            S = np.zeros(nodes)
        kb = _f64(kb) if nold >= 2 else None
        tau = _f64(tau) if nold >= 2 else None
        check(self.lib.fpde_sum_snapshots(self.h, _ptr(S), _ptr(old), nold, OS, nodes, _ptr(tau), _ptr(kb),
                                          1 if dev else 0), "fpde_sum_snapshots")
        return S

    def sum_alg(self, sum_alg, old, tau, kb=None, sum_param=0.0, bs=0, Htmp=None, row2=None, gtj=0.0, gt=0.0,
                alpha=0.0, tstep=0, nodes=None, out=None, sync=True):
        """The reference Sum kernel in history mode sum_alg (0 full, 1 restricted, 2 series
        expansion; fpde_sum). old: (old_size, OS) time-major snapshots (the two newest for
        sum_alg 2); Htmp: (nodes, int(sum_param)) moments (the reference truncates sum_param),
        updated in place. Returns S (into
        `out` when given). With device tensors and sync=False the call is stream-ordered on the
        context's stream and returns after launching."""
        dev = _is_dev(old)
        old = _f64(old)
        nold, OS = old.shape
        nodes = OS if nodes is None else nodes
        if out is not None:
            S = out
        elif dev:
            import torch
            S = torch.zeros(nodes, dtype=torch.float64, device=old.device)
        else:
            S = np.zeros(nodes)
        if sum_alg == 2:
            P = int(sum_param)
            if Htmp is None or tuple(Htmp.shape) != (nodes, P):
                raise ValueError("Htmp must be (nodes, int(sum_param))")
            if not (Htmp.flags["C_CONTIGUOUS"] if not dev else Htmp.is_contiguous()):
                raise ValueError("Htmp must be contiguous")
            row2 = _f64(row2)
        tau = _f64(tau) if tau is not None else None
        kb = _f64(kb) if kb is not None else None
        check(self.lib.fpde_sum(self.h, sum_alg, bs, OS, nodes, _ptr(S), _ptr(old), nold, _ptr(tau), _ptr(Htmp),
                                _ptr(row2), _ptr(kb), float(sum_param), float(gtj), float(gt), float(alpha),
                                int(tstep), (1 if sync else 2) if dev else 0), "fpde_sum")
        return S

    def weights_g(self, p, alpha, time, n0, n1, out=None, sync=True):
        """Generalized-kernel L1 weights (g(t) = t^p) of steps n0..n1 (fpde_weights_g): row
        n - n0 holds kb_0..kb_{n-1} and kkk0 at column n. time: n1 + 2 points (host array or
        device tensor); returns a (n1 - n0 + 1, n1 + 1) array (device tensor for device time)."""
        dev = _is_dev(time)
        time = _f64(time)
        rows, ld = n1 - n0 + 1, n1 + 1
        if out is None:
            if dev:
                import torch
                out = torch.zeros((rows, ld), dtype=torch.float64, device=time.device)
            else:
                out = np.zeros((rows, ld))
        check(self.lib.fpde_weights_g(self.h, float(p), float(alpha), _ptr(time), int(n0), int(n1), _ptr(out),
                                      ld, (1 if sync else 2) if dev else 0), "fpde_weights_g")
        return out

    def _sf_args(self, mat, mc, Tm, x, iw, rs):
        dev = _is_dev(x)
        x = _f64(x)
        lines, m = (1, x.shape[0]) if x.ndim == 1 else x.shape
        mat, mc, Tm = _f64(mat), _f64(mc), _f64(Tm)
        if tuple(mat.shape[-1:]) != (m,) or mat.shape[0] != 3 or tuple(mc.shape) != tuple(mat.shape):
            raise ValueError("mat and mc need shape (3, lines, n+1) (or (3, n+1) for one line)")
        iw = None if iw is None else _f64(iw)
        rs = None if rs is None else _f64(rs)
        return dev, x, lines, m - 1, mat, mc, Tm, iw, rs

    def sf_matvec(self, mat, mc, Tm, x, iw=None, rs=None, space_der=0):
        """The reference's vmul_T (impl 2, toeplitz_mult_alg 0) on one line (x: n+1 values) or a
        batch (x: lines x (n+1)); mat, mc: (3, [lines,] n+1); bitwise the reference's product."""
        dev, x, lines, n, mat, mc, Tm, iw, rs = self._sf_args(mat, mc, Tm, x, iw, rs)
        if dev:
            import torch
            r = torch.empty_like(x)
        else:
            r = np.zeros_like(x)
        check(self.lib.fpde_sf_matvec(self.h, lines, n, _ptr(mat), _ptr(mc), _ptr(Tm), _ptr(iw), _ptr(rs),
                                      int(space_der), _ptr(x), _ptr(r), 1 if dev else 0), "fpde_sf_matvec")
        return r

    def sf_solve(self, mat, mc, Tm, B, x0, thr, maxiter, iw=None, rs=None, space_der=0):
        """solve_mln<1> with vmul_T on every line from the guesses x0: returns (x, iterations)."""
        dev, x, lines, n, mat, mc, Tm, iw, rs = self._sf_args(mat, mc, Tm, x0, iw, rs)
        x = x.clone() if dev else x.copy()
        B = _f64(B)
        if dev:
            import torch
            it = torch.zeros(lines, dtype=torch.int32, device=x.device)
            itp = C.c_void_p(it.data_ptr())
        else:
            it = np.zeros(lines, dtype=np.int32)
            itp = it.ctypes.data_as(C.c_void_p)
        check(self.lib.fpde_sf_solve(self.h, lines, n, _ptr(mat), _ptr(mc), _ptr(Tm), _ptr(iw), _ptr(rs),
                                     int(space_der), _ptr(B), _ptr(x), float(thr), int(maxiter), itp,
                                     1 if dev else 0), "fpde_sf_solve")
        return x, it

    def _sf3d_system(self, dims, mat, mc, Tm, iw, rs, space_der, dev):
        sN, M, K = dims
        V = (sN + 2) * (M + 2) * (K + 2) + 1
        conv = (lambda a: a.contiguous()) if dev else _f64
        mat, mc = conv(mat), conv(mc)
        rows = [conv(t) for t in Tm]
        iw = None if iw is None else conv(iw)
        rs = None if rs is None else conv(rs)
        if tuple(mat.shape) not in ((7, V), (7 * V,)) or tuple(mc.shape) not in ((9, V), (9 * V,)):
            raise ValueError("mat needs 7 x V values and mc 9 x V, V = (sN+2)(M+2)(K+2) + 1")
        if any((t.numel() if dev else t.size) < nl + 1 for t, nl in zip(rows, dims)):
            raise ValueError("Tm[c] needs len_c + 1 values")
        s = Sf3dSystem(sN=sN, M=M, K=K, space_der=int(space_der), mat=_ptr(mat), mc=_ptr(mc), iw=_ptr(iw),
                       rs=_ptr(rs))
        for c in range(3):
            s.Tm[c] = _ptr(rows[c])
        keep = [mat, mc, iw, rs] + rows
        return s, keep, V

    def sf3d_matvec(self, dims, mat, mc, Tm, x, iw=None, rs=None, space_der=0):
        """vmul_T_3d (implicit3d 1) on the V = (sN+2)(M+2)(K+2) + 1 values of x: mat (7, V), mc (9, V),
        Tm three rows (axis sN, _M, K), iw (3, V); bitwise the reference's product. Host arrays or
        CUDA tensors (then the result is a tensor on the same device)."""
        dev = _is_dev(x)
        s, keep, V = self._sf3d_system(dims, mat, mc, Tm, iw, rs, space_der, dev)
        if dev:
            import torch
            x = x.contiguous()
            r = torch.empty_like(x)
        else:
            x = _f64(x)
            r = np.zeros_like(x)
        if (x.numel() if dev else x.size) != V:
            raise ValueError("x needs V values")
        check(self.lib.fpde_sf3d_matvec(self.h, C.byref(s), _ptr(x), _ptr(r), 1 if dev else 0), "fpde_sf3d_matvec")
        return r

    def sf3d_solve(self, dims, mat, mc, Tm, B, x0, thr, maxiter, iw=None, rs=None, space_der=0, exact=False):
        """solve_mln<1> with vmul_T_3d over the V values from x0: returns (x, iterations). exact: the
        reference's sequential dot products (bitwise its iterates); else deterministic tree sums."""
        dev = _is_dev(x0)
        s, keep, V = self._sf3d_system(dims, mat, mc, Tm, iw, rs, space_der, dev)
        if dev:
            x = x0.contiguous().clone()
            B = B.contiguous()
        else:
            x = _f64(x0).copy()
            B = _f64(B)
        it = C.c_int(0)
        check(self.lib.fpde_sf3d_solve(self.h, C.byref(s), _ptr(B), _ptr(x), float(thr), int(maxiter),
                                       1 if exact else 0, C.byref(it), 1 if dev else 0), "fpde_sf3d_solve")
        return x, it.value

    def tridiag_solve(self, a, b, r, om, u, n_lines, N, stride_elem, stride_line, left_kind=0,
                      left_val=None, right_kind=0, right_val=None, dLN=0.0):
        dev = _is_dev(u)
        args = [_f64(x) for x in (a, b, r, om)]
        lv = None if left_val is None else _f64(left_val)
        rv = None if right_val is None else _f64(right_val)
        check(self.lib.fpde_tridiag_solve(self.h, *(_ptr(x) for x in args), _ptr(u), n_lines, N, stride_elem,
                                          stride_line, left_kind, _ptr(lv), right_kind, _ptr(rv), dLN,
                                          1 if dev else 0), "fpde_tridiag_solve")
        return u


class History:
    def __init__(self, ctx, nodes, max_steps, precision=FP64):
        self.ctx, self.nodes = ctx, nodes
        self.h = C.c_void_p()
        check(ctx.lib.fpde_history_create(ctx.h, nodes, max_steps, precision, C.byref(self.h)),
              "fpde_history_create")

    def close(self):
        if self.h:
            self.ctx.lib.fpde_history_destroy(self.h)
            self.h = C.c_void_p()

    def append(self, u):
        u = _f64(u)
        check(self.ctx.lib.fpde_history_append(self.h, _ptr(u), 1 if _is_dev(u) else 0), "fpde_history_append")

    def __len__(self):
        n = C.c_int64()
        check(self.ctx.lib.fpde_history_length(self.h, C.byref(n)), "fpde_history_length")
        return n.value

    def l1_sum(self, kb, tau=None, scale=1.0, out=None):
        kb = np.ascontiguousarray(kb, dtype=np.float64)
        tp = None if tau is None else np.ascontiguousarray(tau, dtype=np.float64)
        if out is None:
            out = np.zeros(self.nodes)
        check(self.ctx.lib.fpde_l1_sum(self.h, _ptr(kb), _ptr(tp), scale, _ptr(out), 1 if _is_dev(out) else 0),
              "fpde_l1_sum")
        return out


class Line:
    """A 1D Caputo line problem advanced on the GPU (fpde_line_*)."""

    def __init__(self, ctx, N, alpha, tau, Da, A, B, Rlap, u0, max_steps, left=(0, 0.0), right=(0, 0.0),
                 dLN=0.0, precision=FP64, block=0, lag_weights=None, theta=0.0, source=None, tuning=None,
                 restrict_eps=0.0, richards=None):
        """lag_weights (max_steps+1 values, w[0] local) replace the Caputo L1 weights (the
        distributed-order equation passes fused weights / tau); theta is the explicit fraction
        of the space operator; source is one row or a (rows, N+1) array of per-step rows;
        restrict_eps > 0 drops the lags from the first one whose kb = w tau / Da is below it
        (the reference's restricted summing); richards = dict(k_form, k_sat, Z, dL, evaporation)
        selects the Richards problem (A, B, Rlap formed from the state every step; they may be
        None)."""
        self.ctx, self.N = ctx, N
        d = LineDesc(N=N, alpha=alpha, tau=tau, Da=Da, left_kind=left[0], left_value=left[1],
                     right_kind=right[0], right_value=right[1], dLN=dLN, precision=precision, block=block,
                     max_steps=max_steps, theta=theta, restrict_eps=restrict_eps)
        self._keep = []
        if lag_weights is not None:
            w = np.ascontiguousarray(lag_weights, dtype=np.float64)
            if len(w) < max_steps + 1:
                raise ValueError("lag_weights needs max_steps + 1 values")
            self._keep.append(w)
            d.lag_weights = w.ctypes.data
        if source is not None:
            src = np.ascontiguousarray(np.atleast_2d(source), dtype=np.float64)
            if src.shape[1] != N + 1:
                raise ValueError("source rows need N + 1 values")
            self._keep.append(src)
            d.source = src.ctypes.data
            d.source_rows = src.shape[0]
        if tuning is not None:
            self._keep.append(tuning)
            d.tuning = C.pointer(tuning)
        if richards is not None:
            z, dl, ev = (np.ascontiguousarray(richards[k], dtype=np.float64) for k in ("Z", "dL", "evaporation"))
            if len(z) < N + 1 or len(dl) < N + 1:
                raise ValueError("richards: Z and dL need N + 1 values")
            r = Richards(k_form=int(richards["k_form"]), k_sat=float(richards["k_sat"]), sZ=z.ctypes.data,
                         evaporation=ev.ctypes.data, evaporation_rows=len(np.atleast_1d(ev)))
            r.dL[0] = dl.ctypes.data
            self._keep.extend([z, dl, ev, r])
            d.richards = C.pointer(r)
        self.desc = d
        arrs = [None if x is None else np.ascontiguousarray(x, dtype=np.float64) for x in (A, B, Rlap, u0)]
        self.h = C.c_void_p()
        check(ctx.lib.fpde_line_create(ctx.h, C.byref(d), *(_ptr(x) for x in arrs), C.byref(self.h)),
              "fpde_line_create")

    def close(self):
        if self.h:
            self.ctx.lib.fpde_line_destroy(self.h)
            self.h = C.c_void_p()

    def reset(self, u0):
        u0 = _f64(u0)
        check(self.ctx.lib.fpde_line_reset(self.h, _ptr(u0), 1 if _is_dev(u0) else 0), "fpde_line_reset")

    def run(self, steps):
        check(self.ctx.lib.fpde_line_run(self.h, steps), "fpde_line_run")

    def state(self, out=None):
        if out is None:
            out = np.zeros(self.N + 1)
        check(self.ctx.lib.fpde_line_get_state(self.h, _ptr(out), 1 if _is_dev(out) else 0), "fpde_line_get_state")
        return out

    def state_ptr(self):
        p = C.c_void_p()
        check(self.ctx.lib.fpde_line_state_ptr(self.h, C.byref(p)), "fpde_line_state_ptr")
        return p.value

    def solve_host(self, u0, steps, out):
        check(self.ctx.lib.fpde_line_solve_host(self.h, _ptr(u0), steps, _ptr(out)), "fpde_line_solve_host")
        return out

    def set_probe(self, every):
        check(self.ctx.lib.fpde_line_set_probe(self.h, every), "fpde_line_set_probe")

    PROBE_HIST, PROBE_FAR, PROBE_SOLVE = 0, 1, 2

    def probe_stats(self, kind):
        ms, b, f, n = C.c_double(), C.c_double(), C.c_double(), C.c_int()
        check(self.ctx.lib.fpde_line_probe_stats(self.h, kind, C.byref(ms), C.byref(b), C.byref(f), C.byref(n)),
              "fpde_line_probe_stats")
        return {"ms": ms.value, "bytes": b.value, "flops": f.value, "count": n.value}

    @property
    def steps_done(self):
        n = C.c_int64()
        check(self.ctx.lib.fpde_line_steps_done(self.h, C.byref(n)), "fpde_line_steps_done")
        return n.value

    def graph_stats(self):
        """fpde_line_graph_stats: (graphs cached now, graphs instantiated since creation)."""
        c, n = C.c_int(), C.c_int64()
        check(self.ctx.lib.fpde_line_graph_stats(self.h, C.byref(c), C.byref(n)), "fpde_line_graph_stats")
        return c.value, n.value

    def step_block(self):
        """fpde_step_block: advance to the next 64-step block boundary; returns the steps run."""
        n = C.c_int()
        check(self.ctx.lib.fpde_step_block(self.h, C.byref(n)), "fpde_step_block")
        return n.value


def _lod3d_desc(dims, alpha, tau, Da, coefA, coefB, coefRlap, max_steps, left_kind, right_kind, dLN, source, bc,
                lag_weights, precision, restrict_eps, series_terms, richards, space_frac, time_steps, weight_rows,
                kernel_power, segments):
    """The fpde_lod3d_desc of Lod3D's arguments, the arrays it points into and the coefficient grids."""
    sN, M, K = dims
    shape = (K + 2, M + 2, sN + 2)
    d = Lod3dDesc(sN=sN, M=M, K=K, alpha=alpha, tau=tau, Da=Da, precision=precision, max_steps=max_steps,
                  restrict_eps=restrict_eps, series_terms=series_terms)
    for q in range(3):
        d.left_kind[q], d.right_kind[q], d.dLN[q] = left_kind[q], right_kind[q], dLN[q]
        d.segments[q] = int(segments[q])
    keep = []

    def rows(x):
        a = np.ascontiguousarray(x, dtype=np.float64)
        if a.shape == shape:
            a = a[None]
        if a.shape[1:] != shape:
            raise ValueError("grid inputs need shape (rows, K+2, M+2, sN+2)")
        keep.append(a)
        return a.ctypes.data, a.shape[0]

    if source is not None:
        d.source, d.source_rows = rows(source)
    if bc is not None:
        d.bc, d.bc_rows = rows(bc)
    if lag_weights is not None:
        w = np.ascontiguousarray(lag_weights, dtype=np.float64)
        if len(w) < max_steps + 1:
            raise ValueError("lag_weights needs max_steps + 1 values")
        keep.append(w)
        d.lag_weights = w.ctypes.data
    if richards is not None:
        arrs = [np.ascontiguousarray(richards[k], dtype=np.float64) for k in ("sZ", "evaporation")]
        dls = [np.ascontiguousarray(x, dtype=np.float64) for x in richards["dL"]]
        if len(arrs[0]) < sN + 2 or any(len(x) < n + 2 for x, n in zip(dls, (sN, M, K))):
            raise ValueError("richards: sZ needs sN+2 values, dL[p] intervals+2")
        keep.extend(arrs + dls)
        r = Richards(k_form=int(richards["k_form"]), k_sat=float(richards["k_sat"]), sZ=arrs[0].ctypes.data,
                     evaporation=arrs[1].ctypes.data, evaporation_rows=len(arrs[1]))
        for q in range(3):
            r.dL[q] = dls[q].ctypes.data
        if richards.get("c0") is not None:            # salt concentration (equation 1)
            c0 = np.ascontiguousarray(richards["c0"], dtype=np.float64)
            if c0.shape != shape:
                raise ValueError("richards: c0 needs the grid's shape")
            keep.append(c0)
            r.salt_c0 = c0.ctypes.data
            r.salt_nu, r.salt_sigma, r.salt_D = (float(richards[k]) for k in ("nu", "sigma", "D"))
        keep.append(r)
        d.richards = C.pointer(r)
    if time_steps is not None:
        ts = np.ascontiguousarray(time_steps, dtype=np.float64)
        if ts.size < max_steps:
            raise ValueError("time_steps needs max_steps values")
        keep.append(ts)
        d.time_steps = ts.ctypes.data
        d.kernel_power = float(kernel_power)
        if weight_rows is not None:
            wr = np.ascontiguousarray(weight_rows, dtype=np.float64)
            if wr.shape != (max_steps, max_steps + 1):
                raise ValueError("weight_rows needs shape (max_steps, max_steps + 1)")
            keep.append(wr)
            d.weight_rows = wr.ctypes.data
    if space_frac is not None:
        f = SpaceFrac(space_der=int(space_frac.get("space_der", 0)), tol=float(space_frac.get("tol", 1e-9)),
                      max_iter=int(space_frac.get("max_iter", 5000)),
                      implicit3d=int(space_frac.get("implicit3d", 0)), exact=int(space_frac.get("exact", 0)))
        for q, nl in enumerate((sN, M, K)):
            tm = np.ascontiguousarray(space_frac["Tm"][q], dtype=np.float64)
            mc = np.ascontiguousarray(space_frac["mc"][q], dtype=np.float64)
            iw = np.ascontiguousarray(space_frac["iw"][q], dtype=np.float64)
            if tm.size < nl + 1 or mc.shape != (3,) + shape or iw.shape != shape:
                raise ValueError("space_frac: Tm[p] needs Nl+1 values, mc[p] (3,)+grid, iw[p] one grid")
            keep.extend([tm, mc, iw])
            f.Tm[q], f.mc[q], f.iw[q] = tm.ctypes.data, mc.ctypes.data, iw.ctypes.data
        keep.append(f)
        d.space_frac = C.pointer(f)
    if coefA is None and richards is not None:
        cs = [None, None, None]
    else:
        cs = [np.ascontiguousarray(x, dtype=np.float64) for x in (coefA, coefB, coefRlap)]
        for c in cs:
            if c.shape != (3,) + shape:
                raise ValueError("coefficient grids need shape (3, K+2, M+2, sN+2)")
    return d, keep, cs


class Lod3D:
    """The 3D LOD step of the reference (fpde_lod3d_*): grids are numpy arrays of shape
    (K+2, M+2, sN+2) (idx = i + j (sN+2) + k (sN+2)(M+2)); coefA/B/Rlap have a leading axis of 3
    passes (0 = sN along i, 1 = _M along j, 2 = K along k)."""

    def __init__(self, ctx, dims, alpha, tau, Da, coefA, coefB, coefRlap, u0, max_steps, left_kind=(0, 0, 0),
                 right_kind=(0, 0, 0), dLN=(0.0, 0.0, 0.0), source=None, bc=None, lag_weights=None,
                 precision=FP64, restrict_eps=0.0, series_terms=0, richards=None, space_frac=None,
                 time_steps=None, weight_rows=None, kernel_power=0.0, segments=(0, 0, 0)):
        """richards: optional dict(k_form, k_sat, sZ, dL=(sdL, dLx, dLy), evaporation) - the
        reference's Richards problem, coefficients formed from the grid every step (coefA/B/Rlap
        may then be None); with c0 (and nu, sigma, D) also the salt concentration (equation 1).
        space_frac: optional dict(space_der, tol, max_iter, Tm=(3 rows), mc=(3 passes x 3 grids),
        iw=(3 grids)) - the reference's implicit space-fractional line solves (impl 2); with
        implicit3d=1 its fully implicit scheme instead (one 3D solve per step; exact=1 for the
        reference's sequential dot products).
        time_steps: optional tau_n of every step (variable steps); weight_rows: optional
        (max_steps, max_steps+1) matrix of the steps' kb_3_cache rows with kkk0 on the diagonal
        (else computed for g(t) = t^kernel_power).
        segments: threads per line of each pass's Thomas sweeps (0 = the built-in rule; see
        autotune_lod3d)."""
        sN, M, K = dims
        self.ctx, self.dims = ctx, dims
        self.shape = (K + 2, M + 2, sN + 2)
        d, keep, cs = _lod3d_desc(dims, alpha, tau, Da, coefA, coefB, coefRlap, max_steps, left_kind, right_kind,
                                  dLN, source, bc, lag_weights, precision, restrict_eps, series_terms, richards,
                                  space_frac, time_steps, weight_rows, kernel_power, segments)
        self._keep = keep
        u0 = np.ascontiguousarray(u0, dtype=np.float64)
        self.h = C.c_void_p()
        check(ctx.lib.fpde_lod3d_create(ctx.h, C.byref(d), *(_ptr(x) for x in cs), _ptr(u0), C.byref(self.h)),
              "fpde_lod3d_create")

    def close(self):
        if self.h:
            self.ctx.lib.fpde_lod3d_destroy(self.h)
            self.h = C.c_void_p()

    def run(self, steps):
        check(self.ctx.lib.fpde_lod3d_run(self.h, steps), "fpde_lod3d_run")

    def state(self, out=None):
        if out is None:
            out = np.zeros(self.shape)
        check(self.ctx.lib.fpde_lod3d_get_state(self.h, _ptr(out), 1 if _is_dev(out) else 0),
              "fpde_lod3d_get_state")
        return out

    def reset(self, u0):
        u0 = _f64(u0)
        check(self.ctx.lib.fpde_lod3d_reset(self.h, _ptr(u0), 1 if _is_dev(u0) else 0), "fpde_lod3d_reset")

    def solve_host(self, u0, steps, out):
        check(self.ctx.lib.fpde_lod3d_solve_host(self.h, _ptr(u0), steps, _ptr(out)), "fpde_lod3d_solve_host")
        return out

    def concentration(self, out=None):
        """The salt concentration grid (Richards problem with richards['c0'])."""
        if out is None:
            out = np.zeros(self.shape)
        check(self.ctx.lib.fpde_lod3d_get_concentration(self.h, _ptr(out), 1 if _is_dev(out) else 0),
              "fpde_lod3d_get_concentration")
        return out

    def sf_iterations(self):
        """Solver iterations of every space-fractional line solve so far."""
        v = C.c_int64()
        check(self.ctx.lib.fpde_lod3d_sf_iterations(self.h, C.byref(v)), "fpde_lod3d_sf_iterations")
        return v.value


class Batch:
    """An ensemble of independent 1D Caputo columns (fpde_batch_*). columns: list of dicts with
    N, alpha, tau, Da, A, B, Rlap, u0 and optional left/right (kind, value), dLN, lag_weights,
    restrict_eps (restricted summing per column)."""

    def __init__(self, ctx, columns, max_steps, precision=FP64):
        self.ctx = ctx
        descs = (ColumnDesc * len(columns))()
        keep = []
        for d, c in zip(descs, columns):
            arrs = [np.ascontiguousarray(c[k], dtype=np.float64) for k in ("A", "B", "Rlap", "u0")]
            keep += arrs
            left, right = c.get("left", (0, 0.0)), c.get("right", (0, 0.0))
            d.N, d.alpha, d.tau, d.Da = c["N"], c.get("alpha", 0.5), c["tau"], c.get("Da", 1.0)
            d.left_kind, d.left_value, d.right_kind, d.right_value = left[0], left[1], right[0], right[1]
            d.dLN = c.get("dLN", 0.0)
            d.restrict_eps = float(c.get("restrict_eps", 0.0))
            d.A, d.B, d.Rlap, d.u0 = (a.ctypes.data for a in arrs)
            if c.get("lag_weights") is not None:
                w = np.ascontiguousarray(c["lag_weights"], dtype=np.float64)
                keep.append(w)
                d.lag_weights = w.ctypes.data
        self.n_cols = len(columns)
        self.h = C.c_void_p()
        check(ctx.lib.fpde_batch_create(ctx.h, descs, len(columns), max_steps, precision, C.byref(self.h)),
              "fpde_batch_create")
        self.layout = []
        for c in range(self.n_cols):
            off, n, tot = C.c_int64(), C.c_int64(), C.c_int64()
            check(ctx.lib.fpde_batch_layout(self.h, c, C.byref(off), C.byref(n), C.byref(tot)), "fpde_batch_layout")
            self.layout.append((off.value, n.value))
            self.total = tot.value

    def close(self):
        if self.h:
            self.ctx.lib.fpde_batch_destroy(self.h)
            self.h = C.c_void_p()

    def run(self, steps):
        check(self.ctx.lib.fpde_batch_run(self.h, steps), "fpde_batch_run")

    def state(self, col=None):
        """Column col's state, or (col None) all columns' states concatenated."""
        if col is None:
            return np.concatenate([self.state(c) for c in range(self.n_cols)])
        out = np.zeros(self.layout[col][1] + 1)
        check(self.ctx.lib.fpde_batch_get_state(self.h, col, _ptr(out), 0), "fpde_batch_get_state")
        return out

    def pack(self, states):
        """Padded device-layout vector from a list of per-column states."""
        v = np.zeros(self.total)
        for (off, n), u in zip(self.layout, states):
            v[off:off + n + 1] = u
        return v

    def unpack(self, v):
        return [v[off:off + n + 1].copy() for off, n in self.layout]

    def reset(self, u_padded=None):
        p = None if u_padded is None else _ptr(_f64(u_padded))
        check(self.ctx.lib.fpde_batch_reset(self.h, p, 1 if (u_padded is not None and _is_dev(u_padded)) else 0),
              "fpde_batch_reset")

    def solve_host(self, u0_padded, steps, out_padded):
        check(self.ctx.lib.fpde_batch_solve_host(self.h, _ptr(u0_padded), steps, _ptr(out_padded)),
              "fpde_batch_solve_host")
        return out_padded


def autotune_lod3d(ctx, dims, alpha, tau, Da, coefA, coefB, coefRlap, u0, max_steps, steps, **kw):
    """fpde_lod3d_autotune: times `steps` steps with each segment count of the Thomas passes and
    returns (segments, ms per step) of the fastest; Lod3D's keyword arguments describe the run."""
    opts = dict(left_kind=(0, 0, 0), right_kind=(0, 0, 0), dLN=(0.0, 0.0, 0.0), source=None, bc=None,
                lag_weights=None, precision=FP64, restrict_eps=0.0, series_terms=0, richards=None, space_frac=None,
                time_steps=None, weight_rows=None, kernel_power=0.0, segments=(0, 0, 0))
    opts.update(kw)
    d, keep, cs = _lod3d_desc(dims, alpha, tau, Da, coefA, coefB, coefRlap, max_steps, opts["left_kind"],
                              opts["right_kind"], opts["dLN"], opts["source"], opts["bc"], opts["lag_weights"],
                              opts["precision"], opts["restrict_eps"], opts["series_terms"], opts["richards"],
                              opts["space_frac"], opts["time_steps"], opts["weight_rows"], opts["kernel_power"],
                              opts["segments"])
    u0 = np.ascontiguousarray(u0, dtype=np.float64)
    seg = (C.c_int * 3)()
    ms = C.c_double()
    check(ctx.lib.fpde_lod3d_autotune(ctx.h, C.byref(d), *(_ptr(x) for x in cs), _ptr(u0), int(steps), seg,
                                      C.byref(ms)), "fpde_lod3d_autotune")
    return tuple(seg), ms.value
