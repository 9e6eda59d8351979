"""B-spline radial basis: breakpoints, knots, quadrature, tables and matrix elements.

Host-side setup of the radial rank. It defines the basis the GPU matvec works in, so
it follows the reference's construction step by step:

* breakpoint sequences: ``pyprop/bspline/breakpointsequences.py:7-130``
  (exponential-linear ``:82-101``);
* continuity and knot sequence: ``pyprop/bspline/BSpline.py:99-168``
  ('zero' continuity drops the end splines, ``:123-126``);
* Gauss-Legendre rule from the Jacobi matrix: ``pyprop/bspline/gausslegendrequadrature.py``;
* global quadrature grid (one rule per breakpoint interval): ``pyprop/bspline/BSpline.py:189-242``;
* B-spline values and derivatives by the Cox-de Boor recursion:
  ``core/transform/bspline/bspline.cpp:25-165``;
* matrix elements ``<B_i| f |B_j^(d)>`` with the transpose sign ``(-1)^d`` for i > j:
  ``core/transform/bspline/bspline.cpp:373-466``.

Nothing here runs per time step.
"""
from __future__ import annotations

import numpy as np

# ---------------------------------------------------------------------------------------
# breakpoint sequences (pyprop/bspline/breakpointsequences.py)
# ---------------------------------------------------------------------------------------


def linear_breakpoints(rmin, rmax, n):
    """``LinearBreakpointSequence`` (breakpointsequences.py:32-38)."""
    return [rmin + (rmax - rmin) * i / float(n - 1) for i in range(n)]


def exponential_breakpoints(rmin, rmax, n, gamma):
    """``ExponentialBreakpointSequence`` (breakpointsequences.py:8-30)."""
    h = rmax - rmin
    return [rmin + h * (np.exp(gamma * float(i - 1) / float(n - 1)) - 1) / (np.exp(gamma) - 1)
            for i in range(1, n + 1)]


def linear_regions_breakpoints(rmin, rmax, n, rcutoff, ratioinner):
    """``LinearBreakpointSequenceRegions`` (breakpointsequences.py:40-49)."""
    innern = int(n * ratioinner)
    outern = n - innern + 1
    return linear_breakpoints(rmin, rcutoff, innern) + linear_breakpoints(rcutoff, rmax, outern)[1:]


def quadratic_linear_breakpoints(rmin, rmax, n, join_point):
    """``QuadraticLinearBreakpointSequence`` (breakpointsequences.py:51-80)."""
    rmin = float(rmin)
    rmax = float(rmax)
    r0 = (rmax * (join_point - 1) + rmin * (n - join_point)) / (2.0 * n - join_point - 1.0)
    alpha = (r0 - rmin) / float(join_point - 1) ** 2
    beta = (rmax - r0) / float(n - join_point)
    xi = [rmin + alpha * (i - 1) ** 2 for i in range(1, join_point)]
    xi += [r0 + beta * (i - join_point) for i in range(join_point, n + 1)]
    return xi


def exponential_linear_breakpoints(rmin, rpartition, rmax, n, gamma):
    """``ExponentialLinearBreakpointSequence`` (breakpointsequences.py:82-101).

    ``n`` exponentially spaced points on [rmin, rpartition], then a linear extension whose
    spacing equals the last inner spacing, up to (and possibly one step past) rmax.
    """
    h = rpartition - rmin
    xi = [rmin + h * (np.exp(gamma * float(i - 1) / float(n - 1)) - 1) / (np.exp(gamma) - 1)
          for i in range(1, n + 1)]
    h = xi[-1] - xi[-2]
    xi += [x for x in np.arange(rpartition + h, rmax + h, h)]
    return xi


def center_exponential_linear_breakpoints(rmin, rpartition, rmax, n, gamma):
    """``CenterExponentialLinearBreakpointSequence`` (breakpointsequences.py:103-130)."""
    center = (rmax + rmin) / 2.0
    h = rpartition - center
    xi = [center + h * (np.exp(gamma * float(i - 1) / float(n - 1)) - 1) / (np.exp(gamma) - 1)
          for i in range(1, n + 1)]
    h = xi[-1] - xi[-2]
    xi += [x for x in np.arange(rpartition + h, rmax + h, h)]
    return [-x for x in reversed(xi[1:])] + xi


def exponential_linear_size_for(rmin, rpartition, rmax, gamma, total):
    """Inner point count ``n`` for which the exponential-linear sequence has ``total``
    breakpoints (searches upwards from 3). Raises if no ``n`` hits ``total`` exactly."""
    for n in range(3, total + 1):
        count = len(exponential_linear_breakpoints(rmin, rpartition, rmax, n, gamma))
        if count == total:
            return n
        if count > total:
            break
    raise ValueError("no exponential-linear inner size gives %d breakpoints" % total)


def exponential_linear_params_for(rmin, rmax, total, gamma=2.0, rpartition=10.0, step=0.25, tries=200):
    """(rpartition, n) giving exactly ``total`` exponential-linear breakpoints.

    Tries ``rpartition``, ``rpartition + step``, ... and for each the inner count ``n``
    (:func:`exponential_linear_size_for`). Deterministic; the chosen values are what a
    config file would record as ``xpartition`` and ``xsize``.
    """
    for t in range(tries):
        rp = rpartition + t * step
        try:
            return rp, exponential_linear_size_for(rmin, rp, rmax, gamma, total)
        except ValueError:
            continue
    raise ValueError("no exponential-linear parameters give %d breakpoints" % total)


# ---------------------------------------------------------------------------------------
# quadrature (pyprop/bspline/gausslegendrequadrature.py)
# ---------------------------------------------------------------------------------------


def gauss_legendre(order):
    """Golub-Welsch Gauss-Legendre rule on [-1, 1]: nodes ascending, weights 2*v0^2."""
    n = np.arange(1, order, dtype=np.float64)
    beta = 1.0 / (2.0 * np.sqrt(1.0 - (2.0 * n) ** -2))
    jac = np.diag(beta, -1) + np.diag(beta, 1)
    e, v = np.linalg.eigh(jac)
    idx = np.argsort(e)
    return e[idx], 2.0 * v[0, idx] ** 2


# ---------------------------------------------------------------------------------------
# the basis
# ---------------------------------------------------------------------------------------


def _safe_div(num, den):
    out = np.zeros(np.broadcast(num, den).shape)
    mask = np.broadcast_to(den != 0, out.shape)
    np.divide(np.broadcast_to(num, out.shape), np.broadcast_to(den, out.shape), out=out, where=mask)
    return out


class BSplineBasis:
    """One B-spline radial basis.

    Attributes mirror the reference object (``core/transform/bspline/bspline.h:22-60``):
    ``NumberOfBSplines``, ``MaxSplineOrder``, breakpoint/continuity/knot sequences and the
    global quadrature grid and weights (``QuadratureGridGlobal`` /
    ``QuadratureWeightsGlobal``).
    """

    def __init__(self, order, breakpoints, continuity="zero", quad_order_additional=0,
                 left_point_continuity=None, right_point_continuity=None):
        self.MaxSplineOrder = k = int(order)
        bps = np.asarray(breakpoints, dtype=np.float64)
        self.breakpoints = bps
        nb = len(bps)
        # continuity sequence (BSpline.py:99-135)
        cont = np.full(nb, k - 1, dtype=int)
        if continuity == "vanilla":
            cont[0] = cont[-1] = 0
        elif continuity == "zero":
            cont[0] = cont[-1] = 1
        elif continuity == "custom":
            cont[0] = left_point_continuity
            cont[-1] = right_point_continuity
        else:
            raise ValueError("Unknown continuity type %r" % (continuity,))
        self.continuity = cont
        # knot sequence (BSpline.py:139-168): multiplicity k - continuity
        self.knots = np.repeat(bps, k - cont)
        self.NumberOfBSplines = len(self.knots) - k
        # quadrature rule: order + quad_order_additional points per breakpoint interval
        self.quad_order = k + int(quad_order_additional)
        nodes, weights = gauss_legendre(self.quad_order)
        a = bps[:-1, None]
        b = bps[1:, None]
        # ScaleAndTranslate (bspline.h:168-171): (x - 1) * (b - a) / 2 + b
        self.grid = ((nodes[None, :] - 1.0) * (b - a) / 2.0 + b).ravel()
        self.weights = ((b - a) / 2.0 * weights[None, :]).ravel()
        self._tables = None

    # -- tables ---------------------------------------------------------------------------
    def _cox_de_boor(self, x, order):
        """All B-splines of ``order`` over the knot sequence at points x: shape (nk-order, nx)."""
        t = self.knots
        x = np.asarray(x, dtype=np.float64)
        B = ((t[:-1, None] <= x[None, :]) & (x[None, :] < t[1:, None])).astype(np.float64)
        for p in range(2, order + 1):
            n = len(t) - p
            left = _safe_div(x[None, :] - t[:n, None], (t[p - 1:p - 1 + n] - t[:n])[:, None]) * B[:n]
            right = _safe_div(t[p:p + n, None] - x[None, :], (t[p:p + n] - t[1:1 + n])[:, None]) * B[1:n + 1]
            B = left + right
        return B

    def _derivative(self, lower, order):
        """d/dx of order-``order`` splines from order-1 values ``lower`` (bspline.cpp:82-108)."""
        t = self.knots
        n = len(t) - order
        c1 = _safe_div(np.full(n, order - 1.0), t[order - 1:order - 1 + n] - t[:n])
        c2 = _safe_div(np.full(n, order - 1.0), t[order:order + n] - t[1:1 + n])
        return c1[:, None] * lower[:n] - c2[:, None] * lower[1:n + 1]

    def tables(self):
        """(B, dB, d2B) at the global quadrature grid, each (N, nquad)."""
        if self._tables is None:
            k = self.MaxSplineOrder
            x = self.grid
            Bkm2 = self._cox_de_boor(x, k - 2)
            Bkm1 = self._cox_de_boor(x, k - 1)
            Bk = self._cox_de_boor(x, k)
            d1 = self._derivative(Bkm1, k)
            d1_km1 = self._derivative(Bkm2, k - 1)
            d2 = self._derivative(d1_km1, k)
            N = self.NumberOfBSplines
            self._tables = (Bk[:N], d1[:N], d2[:N])
        return self._tables

    def evaluate(self, x, coeffs=None):
        """B-spline values at arbitrary points (N, len(x)); with ``coeffs`` the expansion."""
        B = self._cox_de_boor(np.atleast_1d(x), self.MaxSplineOrder)[: self.NumberOfBSplines]
        if coeffs is None:
            return B
        return np.tensordot(coeffs, B, axes=([-1], [0]))

    # -- matrix elements ------------------------------------------------------------------
    def _local(self):
        """Per breakpoint interval m: the k splines nonzero there (index, -1 if dropped) and
        their values and first/second derivatives at the interval's quadrature points.

        Values come from de Boor's triangular recursion (BSPLVB) run on all intervals and
        points at once; the derivatives use the same lower-order formulas as the dense
        tables (bspline.cpp:82-165)."""
        if getattr(self, "_local_cache", None) is None:
            k = self.MaxSplineOrder
            N = self.NumberOfBSplines
            q = self.quad_order
            t = self.knots
            bps = self.breakpoints
            nint = len(bps) - 1
            s_idx = np.searchsorted(t, bps[:-1], side="right") - 1  # knot index of each interval
            x = self.grid.reshape(nint, q)
            # b[p][r]: order-(p+1) splines s-p+r, r = 0..p, at every (interval, point)
            orders = {}
            b = [np.ones_like(x)]
            orders[1] = b
            left = [None] + [x - t[np.clip(s_idx + 1 - j, 0, len(t) - 1)][:, None] for j in range(1, k)]
            right = [None] + [t[np.clip(s_idx + j, 0, len(t) - 1)][:, None] - x for j in range(1, k)]
            for p in range(1, k):
                nb = []
                saved = np.zeros_like(x)
                for r in range(p):
                    den = right[r + 1] + left[p - r]
                    temp = np.divide(b[r], den, out=np.zeros_like(x), where=den != 0)
                    nb.append(saved + right[r + 1] * temp)
                    saved = left[p - r] * temp
                nb.append(saved)
                b = nb
                orders[p + 1] = b

            def deriv(vals_lower, order, first):
                # d/dx of order-`order` splines i = first + r from order-1 splines (same indexing)
                out = []
                for r in range(order):
                    i = first + r
                    acc = np.zeros_like(x)
                    if r - 1 >= 0:  # B_{order-1, i} is index r-1 among order-1 splines starting at first+1
                        den = (t[np.clip(i + order - 1, 0, len(t) - 1)] - t[np.clip(i, 0, len(t) - 1)])
                        c = np.divide(order - 1.0, den, out=np.zeros_like(den, dtype=float), where=den != 0)
                        acc = acc + c[:, None] * vals_lower[r - 1]
                    if r < order - 1:
                        den = (t[np.clip(i + order, 0, len(t) - 1)] - t[np.clip(i + 1, 0, len(t) - 1)])
                        c = np.divide(order - 1.0, den, out=np.zeros_like(den, dtype=float), where=den != 0)
                        acc = acc - c[:, None] * vals_lower[r]
                    out.append(acc)
                return out

            first_k = s_idx - (k - 1)          # first nonzero order-k spline
            vals_k = orders[k]                 # splines first_k + r
            d1 = deriv(orders[k - 1], k, first_k)
            # second derivative: derivative of the order-(k-1) derivatives
            d1_km1 = deriv(orders[k - 2], k - 1, first_k + 1)
            d2 = deriv(d1_km1, k, first_k)
            idx = first_k[:, None] + np.arange(k)[None, :]
            valid = (idx >= 0) & (idx < N)
            idx = np.where(valid, idx, -1)
            loc = []
            for vals in (vals_k, d1, d2):
                L = np.stack(vals, axis=1)  # (nint, k, q)
                L[~valid] = 0.0
                loc.append(L)
            cols = np.arange(nint)[:, None] * q + np.arange(q)[None, :]
            self._local_cache = (idx, valid, cols, loc)
        return self._local_cache

    def band_elements(self, func_values, derivative=0):
        """Matrix elements ``M[i, j] = <B_i | f | d^d B_j>`` for |i - j| < k.

        ``func_values`` is f on the global quadrature grid; a leading batch shape is
        allowed, ``(..., nquad)``. Returns ``(..., N, 2k-1)`` where ``[..., i, (k-1) + (j-i)]``
        holds M[i, j] (zero outside the matrix). For i > j the reference integrates
        ``(-1)^d <B_j| f |d^d B_i>`` (bspline.cpp:379-393); this does the same. The sums run
        interval by interval over the k splines that are nonzero there.
        """
        k = self.MaxSplineOrder
        N = self.NumberOfBSplines
        idx, valid, cols, loc = self._local()
        BL = loc[0]
        DL = loc[derivative]
        f = np.asarray(func_values)
        fw = (f * self.weights)[..., cols]  # (..., nint, q)
        blocks = np.einsum("...mq,maq,mbq->...mab", fw, BL, DL, optimize=True)  # (..., nint, k, k)
        out = np.zeros(f.shape[:-1] + (N, 2 * k - 1), dtype=np.result_type(f, np.float64))
        sign = (-1.0) ** derivative
        # i <= j: <B_i f D_j>; i > j: sign * <B_j f D_i> (the transposed block entry)
        m_i, a_i, b_i = np.meshgrid(np.arange(idx.shape[0]), np.arange(k), np.arange(k), indexing="ij")
        ok = valid[m_i, a_i] & valid[m_i, b_i]
        m_i, a_i, b_i = m_i[ok], a_i[ok], b_i[ok]
        lo = np.minimum(a_i, b_i)
        hi = np.maximum(a_i, b_i)
        vals = blocks[..., m_i, lo, hi]
        vals = np.where(a_i <= b_i, vals, sign * vals)
        rows = idx[m_i, a_i]
        diag = (k - 1) + idx[m_i, b_i] - rows
        flat = rows * (2 * k - 1) + diag
        out2 = out.reshape(f.shape[:-1] + (N * (2 * k - 1),))
        if out2.ndim == 1:
            np.add.at(out2, flat, vals)
        else:
            # one scatter for all leading rows: sum the contributions per target slot with a
            # sparse (contributions x slots) matrix (the same sums as np.add.at row by row)
            import scipy.sparse as sp
            lead = out2.reshape(-1, out2.shape[-1])
            v2 = vals.reshape(-1, vals.shape[-1])
            P = sp.csr_matrix((np.ones(len(flat)), (np.arange(len(flat)), flat)), shape=(len(flat), lead.shape[1]))
            lead += np.asarray((P.T @ v2.T).T)
        return out

    def overlap_band(self):
        """Overlap matrix S as (N, 2k-1) band rows (real)."""
        return self.band_elements(np.ones_like(self.grid), 0)

    def dense(self, band):
        """Expand ``(..., N, 2k-1)`` band rows into dense ``(..., N, N)``."""
        k = self.MaxSplineOrder
        N = self.NumberOfBSplines
        out = np.zeros(band.shape[:-2] + (N, N), dtype=band.dtype)
        for off in range(-(k - 1), k):
            i = np.arange(max(0, -off), min(N, N - off))
            out[..., i, i + off] = band[..., i, (k - 1) + off]
        return out


def bspline_from_config(conf):
    """Build a :class:`BSplineBasis` from a radial representation config section.

    Keys follow ``pyprop/bspline/BSpline.py:15-97``: ``order``, ``bpstype``, ``xmin``,
    ``xmax``, ``xsize``, ``gamma``, ``xpartition``, ``joinpoint``, ``xcutoff``, ``continuity``,
    ``left_point_continuity``, ``right_point_continuity``, ``quad_order_additional``.
    """
    get = conf.get if hasattr(conf, "get") else (lambda key, default=None: getattr(conf, key, default))
    bpstype = get("bpstype")
    if bpstype == "linear":
        bps = linear_breakpoints(get("xmin"), get("xmax"), get("xsize"))
    elif bpstype == "linearregions":
        bps = linear_regions_breakpoints(get("xmin"), get("xmax"), get("xsize"), get("xcutoff"), get("gamma"))
    elif bpstype == "exponential":
        bps = exponential_breakpoints(get("xmin"), get("xmax"), get("xsize"), get("gamma"))
    elif bpstype == "quadraticlinear":
        bps = quadratic_linear_breakpoints(get("xmin"), get("xmax"), get("xsize"), get("joinpoint"))
    elif bpstype == "exponentiallinear":
        bps = exponential_linear_breakpoints(get("xmin"), get("xpartition"), get("xmax"), get("xsize"), get("gamma"))
    elif bpstype == "centerexponentiallinear":
        bps = center_exponential_linear_breakpoints(get("xmin"), get("xpartition"), get("xmax"), get("xsize"),
                                                    get("gamma"))
    else:
        raise NameError("Sequence not recognized: %r" % (bpstype,))
    return BSplineBasis(get("order"), bps, get("continuity", "vanilla"), get("quad_order_additional", 0) or 0,
                        get("left_point_continuity"), get("right_point_continuity"))
