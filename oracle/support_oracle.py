"""Heaviside projection and the self-support / drip constraints on the CPU
(test infrastructure only), restated in FP64 with numpy.

Follows the reference's formulas (grid/Grid.cu:70-300 for H, the overhang,
h-function and drip helper functions; grid/Grid.cu:5529-7156 for the
per-point values and coefficient derivatives; optimization/optimization.cu:
161-183, 243-353 for the projection and its chain rule) and the library's
point rule (level-set crossings on the background lattice, in active
elements, in lattice order, equidistant pick).  Basis derivatives: The NURBS
Book (Piegl and Tiller), algorithm A2.3, on the oracle's knots.
"""
from __future__ import annotations

import math

import numpy as np

ETA = 0.5


def heaviside(s, beta):
    return (np.tanh(beta * ETA) + np.tanh(beta * (s - ETA))) / (np.tanh(beta * ETA) + np.tanh(beta * (1 - ETA)))


def dirac(s, beta):
    t = np.tanh(beta * (s - ETA))
    return beta * (1 - t * t) / (np.tanh(beta * ETA) + np.tanh(beta * (1 - ETA)))


class Spline:
    """The oracle's spline (knots, span rule, coefficients) for point evaluation."""

    def __init__(self, o, order, partition, bmin, bmax, coeff):
        self.k = order
        self.nb = [order + p for p in partition]
        self.U = [o.knots(a, order, partition[a]) for a in range(3)]
        # first knot and step in FP32, as the knot series computes them
        # (grid/Grid.cpp:3263-3287)
        self.kmin, self.step = [], []
        for a in range(3):
            f = np.float32
            mn, mx = f(bmin[a]), f(bmax[a])
            grow = f(f(2.0) * f(mx - mn)) / f(partition[a] + 1)
            mx, mn = f(mx + grow), f(mn - grow)
            self.kmin.append(float(mn))
            self.step.append(float(f(f(mx - mn) / f(partition[a] + 1))))
        self.c = np.asarray(coeff, dtype=np.float64)

    def ders(self, a, x, nd):
        k, p = self.k, self.k - 1
        i = int(math.floor((x - self.kmin[a]) / self.step[a])) + k
        if i < k or i > self.nb[a]:
            return -1, None
        l, U = i - 1, self.U[a]
        ndu = np.zeros((k, k))
        left, right = np.zeros(k), np.zeros(k)
        ndu[0, 0] = 1.0
        for j in range(1, p + 1):
            left[j] = x - U[l + 1 - j]
            right[j] = U[l + j] - x
            saved = 0.0
            for r in range(j):
                ndu[j, r] = right[r + 1] + left[j - r]
                temp = ndu[r, j - 1] / ndu[j, r]
                ndu[r, j] = saved + right[r + 1] * temp
                saved = left[j - r] * temp
            ndu[j, j] = saved
        D = np.zeros((3, k))
        D[0] = ndu[:, p]
        for r in range(p + 1):
            s1, s2 = 0, 1
            aa = np.zeros((2, k))
            aa[0, 0] = 1.0
            for kk in range(1, min(nd, p) + 1):
                d = 0.0
                rk, pk = r - kk, p - kk
                if r >= kk:
                    aa[s2, 0] = aa[s1, 0] / ndu[pk + 1, rk]
                    d = aa[s2, 0] * ndu[rk, pk]
                j1 = 1 if rk >= -1 else -rk
                j2 = kk - 1 if r - 1 <= pk else p - r
                for j in range(j1, j2 + 1):
                    aa[s2, j] = (aa[s1, j] - aa[s1, j - 1]) / ndu[pk + 1, rk + j]
                    d += aa[s2, j] * ndu[rk + j, pk]
                if r <= pk:
                    aa[s2, kk] = -aa[s1, kk - 1] / ndu[pk + 1, r]
                    d += aa[s2, kk] * ndu[r, pk]
                D[kk, r] = d
                s1, s2 = s2, s1
        f = float(p)
        for kk in range(1, nd + 1):
            D[kk] *= f
            f *= (p - kk)
        return i - k, D

    def idx(self, i0, r, q, t):
        return (i0[0] + r) + self.nb[0] * ((i0[1] + q) + self.nb[1] * (i0[2] + t))

    def value(self, x, outside):
        i0, D = [], []
        for a in range(3):
            i, d = self.ders(a, x[a], 0)
            if i < 0:
                return outside
            i0.append(i)
            D.append(d)
        v = 0.0
        for r in range(self.k):
            for q in range(self.k):
                for t in range(self.k):
                    v += self.c[self.idx(i0, r, q, t)] * D[0][0, r] * D[1][0, q] * D[2][0, t]
        return v


def surface_points(o, spl, dims, h, eactive, lattice, max_points):
    """(candidates, points [n][3]) by the library's lattice rule."""
    n = lattice + 2
    bmax = np.array(dims, dtype=np.float64) * h
    e = bmax / lattice
    org = -e
    lat = np.zeros(n ** 3)
    for z in range(n):
        for y in range(n):
            for x in range(n):
                p = org + (np.array([x, y, z]) + 0.5) * e
                inside = np.all(p >= 0) and np.all(p <= bmax)
                lat[x + n * (y + n * z)] = spl.value(p, -0.2) - 0.5 if inside else -0.5

    def pos(i):
        return org + (np.array([i % n, (i // n) % n, i // (n * n)]) + 0.5) * e

    cand = []
    for nid in range(n ** 3):
        c = (nid % n, (nid // n) % n, nid // (n * n))
        for a in range(3):
            if c[a] + 1 >= n:
                continue
            nid1 = nid + (1, n, n * n)[a]
            v0, v1 = lat[nid], lat[nid1]
            if (v0 < 0) == (v1 < 0):
                continue
            t = -v0 / (v1 - v0)
            p0, p1 = pos(nid), pos(nid1)
            p = p0 + t * (p1 - p0)
            if not (np.all(p >= 0) and np.all(p <= bmax)):
                continue
            ec = [min(max(int(math.floor(p[k] / h)), 0), dims[k] - 1) for k in range(3)]
            if eactive[ec[0] + dims[0] * (ec[1] + dims[1] * ec[2])]:
                cand.append(p)
    count = len(cand)
    if count > max_points:
        step = count / (max_points - 1)
        picks = [min(int(k * step), count - 1) for k in range(max_points)]
    else:
        picks = list(range(count))
    return count, np.array([cand[i] for i in picks]).reshape(-1, 3)


def _fh(x, c): return c * (x - 1) ** 2 if x >= 1 else 0.0
def _dfh(x, c): return 2 * c * (x - 1) if x >= 1 else 0.0
def _foh(x, c): return 1 / (1 + math.exp(-(x - 1.5) / c)) + 1
def _dfoh(x, c):
    ee = math.exp(-(x - 1.5) / c)
    return 1 / (1 + ee) / (1 + ee) / c * ee
def _amax1(x, b, s): return s * x * x / (1 + math.exp(b * x))
def _damax1(x, b, s):
    ee = 1 + math.exp(b * x)
    return s * (2 * x - x * x * b) / ee + s * x * x * b / ee / ee
def _amax2(x, b, s): return s * x * x / (1 + math.exp(-b * x))
def _damax2(x, b, s):
    ee = 1 + math.exp(-b * x)
    return s * (2 * x + x * x * b) / ee - s * x * x * b / ee / ee
def _drip_up(x, mu, tol):
    return 1 / (1 + math.exp(-(x - 1.2) * mu)) if tol > 0.5 * math.pi else 1 / (1 + math.exp(mu * (x + 1.2)))
def _ddrip_up(x, mu, tol):
    if tol > 0.5 * math.pi:
        ee = math.exp(-(x - 1.2) * mu)
        return 1 / (1 + ee) / (1 + ee) * mu * ee
    ee = math.exp(mu * (x + 1.2))
    return -mu * ee / (1 + ee) / (1 + ee)


def constraints(spl, pts, opts, beta, nc):
    """Values and coefficient gradients for the given points (the GPU's point
    set), following the reference's per-point formulas."""
    o = dict(opts)
    P = dict(p_norm=o.get("p_norm") or 8.0, hc=o.get("hfunction_c") or 10.0, sc=o.get("sigmoid_c") or 0.09,
             db=o.get("drip_beta") or 128.0, mu=o.get("drip_mu") or 32.0,
             da=o.get("drip_angle") or 160.0 / 180.0 * math.pi, al=o.get("drip_alpha") or 4.0,
             ds=o.get("drip_beta_scale") or 10.0)
    ssm, dm, ver, quirks = o["ss_mode"], o["drip_mode"], o.get("drip_version", 0), o.get("reference_quirks", 0)
    cp, cd = math.cos(o["print_angle"] * math.pi), math.cos(P["da"])
    npts, k = len(pts), spl.k
    info = []
    votes = 0.0
    for p in pts:
        i0, D = [], []
        for a in range(3):
            i, d = spl.ders(a, p[a], 2)
            i0.append(i)
            D.append(d)
        g, H = np.zeros(3), np.zeros(3)
        if min(i0) >= 0:
            for r in range(k):
                for q in range(k):
                    for t in range(k):
                        c = spl.c[spl.idx(i0, r, q, t)]
                        g += c * np.array([D[0][1, r] * D[1][0, q] * D[2][0, t], D[0][0, r] * D[1][1, q] * D[2][0, t],
                                           D[0][0, r] * D[1][0, q] * D[2][1, t]])
                        H += c * np.array([D[0][2, r] * D[1][0, q] * D[2][0, t], D[0][0, r] * D[1][2, q] * D[2][0, t],
                                           D[0][1, r] * D[1][1, q] * D[2][0, t]])
        sv = spl.value(p + 1e-3 * g, -0.1)
        votes += 1.0 if heaviside(sv, beta) < 0.5 else -1.0
        info.append((i0, D, g, H))
    flip = votes < 0
    direction = 1.0 if votes > 0 else -1.0
    ssv, dripv, down = np.zeros(npts), np.zeros(npts), np.zeros(npts)
    gss, gdrip = np.zeros(nc), np.zeros(nc)
    contrib_ss, contrib_drip = [], []
    for m, (i0, D, g, H) in enumerate(info):
        n = -g if flip else g
        nn = float(np.linalg.norm(n))
        inner = n[2] / nn / cp
        isdown = n[2] < 0
        down[m] = 1.0 if isdown else 0.0
        if ssm == 0: ssv[m] = inner ** P["p_norm"] if isdown else 0.0
        elif ssm == 1: ssv[m] = inner ** P["p_norm"]
        elif ssm == 2: ssv[m] = _fh(inner, P["hc"]) if isdown else 0.0
        elif ssm == 3: ssv[m] = _fh(inner, P["hc"])
        elif ssm == 4: ssv[m] = _foh(inner, P["sc"]) if isdown else 0.0
        else: ssv[m] = _foh(inner, P["sc"])
        if ssm == 0: dss = P["p_norm"] * inner ** (P["p_norm"] - 1) if isdown else 0.0
        elif ssm == 1: dss = P["p_norm"] * inner ** (P["p_norm"] - 1)
        elif ssm == 2: dss = _dfh(inner, P["hc"]) if isdown else 0.0
        elif ssm == 3: dss = _dfh(inner, P["hc"])
        elif ssm == 4: dss = _dfoh(inner, P["sc"]) if isdown else 0.0
        else: dss = _dfoh(inner, P["sc"])
        drip_on = dm == 7 or (dm == 6 and isdown)
        hinner = n[2] / nn / cd
        i1, i2 = H[0], H[0] * H[1] - H[2] * H[2]
        tq1, tq2 = _amax1(i1, P["db"], P["ds"]), _amax2(i2, P["db"], P["ds"])
        dtq1, dtq2 = _damax1(i1, P["db"], P["ds"]), _damax2(i2, P["db"], P["ds"])
        gx, gy = n[0] / n[2], n[1] / n[2]
        g_ = math.exp(-P["al"] * gx * gx - P["al"] * gy * gy)
        h_, dh_ = _drip_up(hinner, P["mu"], P["da"]), _ddrip_up(hinner, P["mu"], P["da"])
        if drip_on:
            dripv[m] = (g_ if ver == 1 else h_) * tq1 * tq2
        if min(i0) < 0:
            continue
        acc = np.zeros(4)
        for r in range(k):
            for q in range(k):
                for t in range(k):
                    ci = spl.idx(i0, r, q, t)
                    dn = direction * np.array([D[0][1, r] * D[1][0, q] * D[2][0, t], D[0][0, r] * D[1][1, q] * D[2][0, t],
                                               D[0][0, r] * D[1][0, q] * D[2][1, t]])
                    dnn = float(n @ dn) / nn
                    up_p = dn[2] * nn - n[2] * dnn
                    contrib_ss.append((ci, dss * (up_p / (nn * nn * cp))))
                    dv = 0.0
                    if drip_on:
                        hd = up_p / (nn * nn * cd)
                        d00 = D[0][2, r] * D[1][0, q] * D[2][0, t]
                        d11 = D[0][0, r] * D[1][2, q] * D[2][0, t]
                        d01 = D[0][1, r] * D[1][1, q] * D[2][0, t]
                        d10 = d01
                        gdx = (dn[0] * n[2] - n[0] * dn[2]) / (n[2] * n[2])
                        gdy = (dn[1] * n[2] - n[1] * dn[2]) / (n[2] * n[2])
                        if quirks:
                            acc += [d00, d11, d01, d10]
                            d00, d11, d01, d10 = acc
                            gdx, gdy = gdy, 0.0
                        di1 = d00
                        di2 = d00 * H[1] + H[0] * d11 - d01 * H[2] - H[2] * d10
                        dg = (-2 * P["al"] * gx * gdx - 2 * P["al"] * gy * gdy) * g_
                        if ver == 1:
                            dv = (dg * hd if quirks else dg) * tq1 * tq2 + g_ * dtq1 * di1 * tq2 + g_ * tq1 * dtq2 * di2
                        else:
                            dv = dh_ * hd * tq1 * tq2 + h_ * dtq1 * di1 * tq2 + h_ * tq1 * dtq2 * di2
                    contrib_drip.append((ci, dv))
    for ci, v in contrib_ss:
        gss[ci] += v
    for ci, v in contrib_drip:
        gdrip[ci] += v
    cnt_ss = down.sum() if ssm % 2 == 0 else npts
    cnt_drip = down.sum() if dm % 2 == 0 else npts
    ss = 0.0
    if cnt_ss > 0:
        ss = (ssv.sum() / cnt_ss) ** (1 / P["p_norm"]) - 1 if ssm <= 1 else ssv.sum() / cnt_ss
    drip = 0.0
    if cnt_drip > 0:
        drip = (dripv.sum() / cnt_drip) ** (1 / P["p_norm"]) - 1 if dm <= 1 else dripv.sum() / cnt_drip
    gss = gss / cnt_ss if cnt_ss > 0 else gss * 0
    gdrip = gdrip / cnt_drip if cnt_drip > 0 else gdrip * 0
    normals = np.array([(-g if flip else g) for (_, _, g, _) in info]).reshape(-1, 3)
    return dict(ss=ss, drip=drip, gss=gss, gdrip=gdrip, flipped=bool(flip), down=int(down.sum()), normals=normals)
