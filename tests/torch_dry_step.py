"""FP64 restatement of the dry RKHEVI step in PyTorch (CPU), for tests.

Its reverse-mode automatic differentiation is the CPU adjoint the GPU's
hand-written adjoint kernels are compared with.  The restatement follows the
oracle's operators (which are pinned to the reference) with the fields held
as 2-D tensors: cells [layer][cell], interfaces [level][cell], edges
[layer][edge], tangential vorticity [level][edge], rhombus vorticity
[layer][edge], triangles [layer][triangle]; the reference's vector and curl
layouts are converted at the boundary.  Values agree with the oracle to
rounding (summation order of the vectorised gathers), checked in
test_torch_adjoint.py.

Scope: the dry build (one constituent); diffusion, radiation and surface
fluxes off, as in every benchmark configuration.
"""
import math

import numpy as np
import torch

T0 = torch.float64
C_D_V, C_D_P, R_D = 717.942189, 1005.0, 287.057811
N_PENT = 12


class DryGrid:
    """the grid tables of one Model in 2-D tensor form"""

    def __init__(self, m):
        lay = m.layout
        g, dg = m.grid, m.dualgrid
        self.nc, self.ne, self.nt, self.nl = lay.nc, lay.ne, lay.nt, lay.nl
        nc, ne, nt, L = self.nc, self.ne, self.nt, self.nl
        self.n_oro = int(g["no_of_oro_layers"][0])
        self.radius = float(g["radius"][0])
        vpl, dpl = nc + ne, ne + nt
        t = lambda a: torch.tensor(np.ascontiguousarray(a), dtype=T0)
        ti = lambda a: torch.tensor(np.ascontiguousarray(a), dtype=torch.long)

        def vsplit(a):
            a = np.asarray(a)
            v = np.stack([a[k * vpl:k * vpl + nc] for k in range(L + 1)])
            h = np.stack([a[nc + l * vpl:(l + 1) * vpl] for l in range(L)])
            return t(v), t(h)

        self.nd_v, self.nd_h = vsplit(g["normal_distance"])
        self.area_v, self.area_h = vsplit(g["area"])
        self.zvec_v, self.z_h = vsplit(g["z_vector"])
        self.ebgg_v, self.ebgg_h = vsplit(g["exner_bg_grad"])
        _, self.slope_h = vsplit(g["slope"])
        r = lambda name: t(np.asarray(g[name]).reshape(L, nc))
        self.volume, self.z_scalar = r("volume"), r("z_scalar")
        self.theta_bg, self.exner_bg = r("theta_v_bg"), r("exner_bg")
        self.ipw = t(np.asarray(g["inner_product_weights"]).reshape(L, nc, 8))
        self.adj = ti(np.asarray(g["adjacent_vector_indices_h"]).reshape(nc, 6))
        self.sign = t(np.asarray(g["adjacent_signs_h"], dtype=np.float64).reshape(nc, 6))
        self.frm, self.to = ti(g["from_index"]), ti(g["to_index"])
        self.tw = t(np.asarray(g["trsk_weights"]).reshape(ne, 10))
        # unused pentagon slots are masked below; clamp them to valid edges
        self.ti = ti(np.clip(np.asarray(g["trsk_indices"]).reshape(ne, 10), 0, ne - 1))
        self.tm = ti(np.clip(np.asarray(g["trsk_modified_curl_indices"]).reshape(ne, 10), 0, ne - 1))
        self.rw = t(np.asarray(g["density_to_rhombi_weights"]).reshape(ne, 4))
        self.ri = ti(np.asarray(g["density_to_rhombi_indices"]).reshape(ne, 4))
        da, dz = np.asarray(dg["area"]), np.asarray(dg["z_vector"])
        self.darea_h = t(np.stack([da[k * dpl:k * dpl + ne] for k in range(L + 1)]))
        self.darea_t = t(np.stack([da[ne + l * dpl:ne + l * dpl + nt] for l in range(L)]))
        self.dz_t = t(np.stack([dz[ne + l * dpl:ne + l * dpl + nt] for l in range(L)]))
        fv = np.asarray(dg["f_vec"])
        self.f_h, self.f_r = t(fv[:ne]), t(fv[ne:2 * ne])
        self.vi = ti(np.asarray(dg["vorticity_indices_triangles"]).reshape(nt, 3))
        self.vs = t(np.asarray(dg["vorticity_signs_triangles"], dtype=np.float64).reshape(nt, 3))
        self.dfrom, self.dto = ti(dg["from_index"]), ti(dg["to_index"])
        # z_vector as calc_pot_vort reads it, past its end into gravity_potential, gravity_m
        zext = np.concatenate([np.asarray(g["z_vector"]), np.asarray(g["gravity_potential"]),
                               np.asarray(g["gravity_m"])])
        ns = L * nc
        h = np.arange(ne)
        fr, to = np.asarray(g["from_index"]), np.asarray(g["to_index"])
        self.pvz0 = t(zext[0] - zext[ns + h])
        self.pvz1 = t(zext[ns + h] - zext[ns + vpl + h])
        self.pvz2 = t(0.5 * (zext[L * vpl + fr] + zext[L * vpl + to]) - zext[ns + (L - 1) * vpl + h])
        self.pvz3 = t(zext[ns + (L - 2) * vpl + h] - zext[ns + (L - 1) * vpl + h])
        self.n_edges = torch.where(torch.arange(nc) < N_PENT, 5, 6)
        # Klemp damping denominators' coefficients per inner interface
        self.zv_inner = self.zvec_v[1:L]
        self.toa = float(np.asarray(g["z_vector"])[0])


# ------------------------------------------------------------------ operators
def grad(G, f):
    """gradient_operators.c:66-74 -> (vertical [L+1, Nc] inner levels, horizontal [L, Ne])"""
    L = G.nl
    gv = torch.zeros(L + 1, G.nc, dtype=T0)
    gv[1:L] = (f[:L - 1] - f[1:]) / G.nd_v[1:L]
    gh = (f[:, G.to] - f[:, G.frm]) / G.nd_h
    gh = cov_to_con(G, gv, gh)
    return gv, gh


def remap(G, fv, l):
    """averaging.c:14-39 at layer l for every edge"""
    fr, to = G.frm, G.to
    c = G.ipw[l, fr, 6] * fv[l, fr]
    c = c + G.ipw[l, to, 6] * fv[l, to]
    if l < G.nl - 1:
        c = c + G.ipw[l, fr, 7] * fv[l + 1, fr]
        c = c + G.ipw[l, to, 7] * fv[l + 1, to]
    return 0.5 * c


def cov_to_con(G, fv, fh):
    rows = []
    for l in range(G.nl):
        if l >= G.nl - G.n_oro:
            rows.append(fh[l] + (-G.slope_h[l]) * remap(G, fv, l))
        else:
            rows.append(fh[l])
    return torch.stack(rows)


def hor_cov(G, u, w, l):
    if l >= G.nl - G.n_oro:
        return u[l] + G.slope_h[l] * remap(G, w, l)
    return u[l]


def stv_h(G, s, vh):
    return (0.5 * (s[:, G.to] + s[:, G.frm])) * vh


def stv_v(G, s, vv):
    out = torch.zeros_like(vv)
    out[1:G.nl] = (0.5 * (s[:G.nl - 1] + s[1:])) * vv[1:G.nl]
    return out


def inner(G, u, w):
    L = G.nl
    acc = torch.zeros(L, G.nc, dtype=T0)
    for j in range(6):
        mask = (G.n_edges > j).to(T0)
        ue = u[:, G.adj[:, j]]
        acc = acc + mask * (G.ipw[:, :, j] * ue * ue)
    acc = acc + G.ipw[:, :, 6] * w[:L] * w[:L]
    acc = acc + G.ipw[:, :, 7] * w[1:] * w[1:]
    return acc


def tri_vort(G, u):
    L = G.nl
    rows = []
    for l in range(L):
        acc = torch.zeros(G.nt, dtype=T0)
        for j in range(3):
            e = G.vi[:, j]
            vel = u[l, e]
            rescale = torch.ones(G.nt, dtype=T0)
            if l >= L - G.n_oro:
                zt = G.dz_t[l]
                zh = G.z_h[l, e]
                rescale = (G.radius + zt) / (G.radius + zh)
                dz = zt - zh
                lo = torch.where(dz > 0, l - 1, l - 1 if l == L - 1 else l + 1)
                ulo = u[lo, e]
                vgrad = (u[l, e] - ulo) / (zh - G.z_h[lo, e])
                vel = vel + dz * vgrad
            acc = acc + rescale * G.nd_h[l, e] * G.vs[:, j] * vel
        rows.append(acc / G.darea_t[l])
    return torch.stack(rows)


def pot_vort(G, u, w, rho):
    """vorticities.c:18-85 -> tangential [L+1, Ne], rhombus [L, Ne]"""
    L, nc = G.nl, G.nc
    fr, to = G.frm, G.to
    tri = tri_vort(G, u)
    zh_rows = []
    for k in range(L + 1):
        kk = max(k, 1)
        ia = 1.0 / G.darea_h[kk]
        if kk == L:
            rel = ia * G.nd_h[kk - 1] * hor_cov(G, u, w, kk - 1)
        else:
            rel = ia * (-G.nd_h[kk] * hor_cov(G, u, w, kk) + G.nd_v[kk, fr] * w[kk, fr]
                        + G.nd_h[kk - 1] * hor_cov(G, u, w, kk - 1) - G.nd_v[kk, to] * w[kk, to])
        if k == 0:
            top = 0.5 * (rho[0, fr] + rho[0, to])
            below = 0.5 * (rho[1, fr] + rho[1, to])
            dens = top + (top - below) / G.pvz1 * G.pvz0
        elif k == L:
            low = 0.5 * (rho[L - 1, fr] + rho[L - 1, to])
            above = 0.5 * (rho[L - 2, fr] + rho[L - 2, to])
            dens = low + (above - low) / G.pvz3 * G.pvz2
        else:
            dens = 0.25 * (rho[k - 1, fr] + rho[k - 1, to] + rho[k, fr] + rho[k, to])
        zh_rows.append((rel + G.f_h) / dens)
    zv_rows = []
    for l in range(L):
        af, at = G.darea_t[l, G.dfrom], G.darea_t[l, G.dto]
        rel = (af * tri[l, G.dfrom] + at * tri[l, G.dto]) / (af + at)
        dens = torch.zeros(G.ne, dtype=T0)
        for j in range(4):
            dens = dens + G.rw[:, j] * rho[l, G.ri[:, j]]
        zv_rows.append((rel + G.f_r) / dens)
    return torch.stack(zh_rows), torch.stack(zv_rows)


def vflux(G, fv, fh, zh, zv):
    """vorticity_flux.c:16-187 -> (vertical [L+1, Nc], horizontal [L, Ne])"""
    L = G.nl
    fr, to = G.frm, G.to
    pent_f, pent_t = (fr < N_PENT), (to < N_PENT)
    out_h = []
    for l in range(L):
        mf, pv = fh[l], zv[l]
        acc = torch.zeros(G.ne, dtype=T0)
        for j in range(10):
            term = G.tw[:, j] * mf[G.ti[:, j]] * pv[G.tm[:, j]]
            if j in (2, 7):
                half = G.tw[:, j] * mf[G.ti[:, j]] * 0.5 * (pv[G.tm[:, j]] + pv)
                pent = pent_f if j == 2 else pent_t
                term = torch.where(pent, term, half)
            if j == 4:
                term = torch.where(pent_f, torch.zeros_like(term), term)
            if j == 9:
                term = torch.where(pent_t, torch.zeros_like(term), term)
            acc = acc + term
        zt, zb = zh[l], zh[l + 1]
        acc = acc - 0.5 * G.ipw[l, fr, 6] * fv[l, fr] * zt
        acc = acc - 0.5 * G.ipw[l, to, 6] * fv[l, to] * zt
        acc = acc - 0.5 * G.ipw[l, fr, 7] * fv[l + 1, fr] * zb
        acc = acc - 0.5 * G.ipw[l, to, 7] * fv[l + 1, to] * zb
        out_h.append(acc)
    out_v = []
    for k in range(L + 1):
        vw = 1.0 if k in (0, L) else 0.5
        acc = torch.zeros(G.nc, dtype=T0)
        for j in range(6):
            mask = (G.n_edges > j).to(T0)
            a = G.adj[:, j]
            if k >= 1:
                acc = acc + mask * (vw * G.ipw[k - 1, :, j] * fh[k - 1, a] * zh[k, a])
            if k <= L - 1:
                acc = acc + mask * (vw * G.ipw[k, :, j] * fh[k, a] * zh[k, a])
        out_v.append(acc)
    return torch.stack(out_v), torch.stack(out_h)


def contra_corr(G, fh, layer):
    """averaging.c:41-95 for every cell"""
    L = G.nl
    r = torch.zeros(G.nc, dtype=T0)
    if layer < L - G.n_oro:
        return r
    layers = [layer] if layer == L - G.n_oro else [layer - 1, layer]
    for ll in layers:
        for j in range(6):
            mask = (G.n_edges > j).to(T0)
            a = G.adj[:, j]
            r = r + mask * (-0.5 * G.ipw[ll, :, j] * G.slope_h[ll, a] * fh[ll, a])
    return r


def divv_h(G, fh):
    """divergences.c:14-64"""
    L, n_oro = G.nl, G.n_oro
    rows = []
    for l in range(L):
        comp_h = torch.zeros(G.nc, dtype=T0)
        for j in range(6):
            mask = (G.n_edges > j).to(T0)
            a = G.adj[:, j]
            comp_h = comp_h + mask * (fh[l, a] * G.sign[:, j] * G.area_h[l, a])
        if l == L - n_oro - 1:
            comp_v = -contra_corr(G, fh, l + 1) * G.area_v[l + 1]
        elif l == L - 1:
            comp_v = contra_corr(G, fh, l) * G.area_v[l]
        elif l > L - n_oro - 1:
            comp_v = contra_corr(G, fh, l) * G.area_v[l] - contra_corr(G, fh, l + 1) * G.area_v[l + 1]
        else:
            comp_v = 0.0
        rows.append(1.0 / G.volume[l] * (comp_h + comp_v))
    return torch.stack(rows)


# ------------------------------------------------------------------ the step
class DryStep:
    def __init__(self, m, dt):
        self.G = DryGrid(m)
        self.dt = dt
        c = m.config
        self.iw = float(c["impl_thermo_weight"][0])
        G = self.G
        damp_start = float(c["damping_start_height_over_toa"][0]) * G.toa
        cmax = float(c["damping_coeff_max"][0])
        zad = G.zv_inner - damp_start
        dc = torch.where(zad < 0, torch.zeros_like(zad),
                         cmax * torch.sin(0.5 * math.pi * zad / (G.toa - damp_start)) ** 2)
        self.dden = 1.0 + dt * dc
        self.fv_bounds = None

    def pgrad(self, s):
        G = self.G
        gv, gh = grad(G, s["ep"])
        sfac = C_D_P * (G.theta_bg + s["tp"])
        nl_v, nl_h = stv_v(G, sfac, gv), stv_h(G, sfac, gh)
        lfac = C_D_P * s["tp"]
        l_v, l_h = stv_v(G, lfac, G.ebgg_v), stv_h(G, lfac, G.ebgg_h)
        return nl_v + l_v, nl_h + l_h

    def advection(self, s):
        G = self.G
        fh = stv_h(G, s["rho"], s["u"])
        fv = stv_v(G, s["rho"], s["w"])
        fv = torch.cat([self.fv_bounds[0:1], fv[1:G.nl], self.fv_bounds[1:2]])
        zh, zv = pot_vort(G, s["u"], s["w"], s["rho"])
        pvt_v, pvt_h = vflux(G, fv, fh, zh, zv)
        v2 = inner(G, s["u"], s["w"])
        v2g_v, v2g_h = grad(G, v2)
        return (pvt_v, pvt_h), (v2g_v, v2g_h)

    def scalar(self, rho, rt, u):
        G = self.G
        fh = stv_h(G, rho, u)
        d = divv_h(G, fh)
        theta = rt / rho
        ft = stv_h(G, theta, fh)
        dt_ = divv_h(G, ft)
        return -d, -dt_

    def waves(self, so, sn, st_rho, st_rt, st_w, rk):
        G, dt, iw = self.G, self.dt, self.iw
        L = G.nl
        vol = G.volume
        ro, rto = so["rho"], so["rt"]
        if rk == 0:
            alpha = -rto / (ro * ro) / vol
            beta = 1.0 / ro / vol
            gam = R_D / (C_D_V * rto) * (G.exner_bg + so["ep"]) / vol
        else:
            rn, rtn = sn["rho"], sn["rt"]
            ao, bo = -rto / (ro * ro), 1.0 / ro
            go = R_D / (C_D_V * rto) * (G.exner_bg + so["ep"])
            an, bn = -rtn / (rn * rn), 1.0 / rn
            gn = R_D / (C_D_V * rtn) * (G.exner_bg + sn["ep"])
            alpha = (0.5 * ao + 0.5 * an) / vol
            beta = (0.5 * bo + 0.5 * bn) / vol
            gam = (0.5 * go + 0.5 * gn) / vol
        rexp = ro + dt * st_rho
        rtexp = rto + dt * st_rt
        tpexp = so["tp"] + dt * vol * (alpha * st_rho + beta * st_rt)
        epexp = so["ep"] + dt * vol * gam * st_rt
        thl = sn["rt"] / sn["rho"]
        rho_io = 0.5 * (ro[:-1] + ro[1:])
        rho_ie = 0.5 * (rexp[:-1] + rexp[1:])
        th = 0.5 * (thl[:-1] + thl[1:])
        dz = G.z_scalar[:-1] - G.z_scalar[1:]
        dpi = G.exner_bg[:-1] - G.exner_bg[1:]
        wo = so["w"][1:L]
        K1, K2 = iw * dt * dt * C_D_P, iw * dt * C_D_P
        d = (-(th * th) * (gam[:-1] + gam[1:]) + 0.5 * dpi * (alpha[1:] - alpha[:-1] + th * (beta[1:] - beta[:-1]))
             - dz / (K1 * rho_io) * (2.0 / G.area_v[1:L] + dt * wo * 0.5 * (-1.0 / vol[:-1] + 1.0 / vol[1:])))
        r = (-(wo + dt * st_w[1:L]) * dz / K1 + th * (epexp[:-1] - epexp[1:]) / dt
             + 0.5 / dt * (tpexp[:-1] + tpexp[1:]) * dpi - dz / K1 * wo * rho_ie / rho_io)
        c = (th[1:] * gam[1:-1] * th[:-1] + 0.5 * dpi[1:] * (alpha[1:-1] + beta[1:-1] * th[:-1])
             - dz[1:] / K2 * 0.5 * wo[1:] / (vol[1:-1] * rho_io[1:]))
        e = (th[:-1] * gam[1:-1] * th[1:] - 0.5 * dpi[:-1] * (alpha[1:-1] + beta[1:-1] * th[1:])
             + dz[:-1] / K2 * 0.5 * wo[:-1] / (vol[1:-1] * rho_io[:-1]))
        n = L - 1
        ep, rp = [None] * n, [None] * n
        ep[0] = e[0] / d[0]
        rp[0] = r[0] / d[0]
        for j in range(1, n):
            den = d[j] - ep[j - 1] * c[j - 1]
            if j < n - 1:
                ep[j] = e[j] / den
            rp[j] = (r[j] - rp[j - 1] * c[j - 1]) / den
        x = [None] * n
        x[n - 1] = rp[n - 1]
        for j in range(n - 2, -1, -1):
            x[j] = rp[j] - ep[j] * x[j + 1]
        sol = torch.stack(x) / self.dden
        zero = torch.zeros(1, G.nc, dtype=T0)
        s_up = torch.cat([zero, sol])      # sol of the interface above each layer (0 at the TOA)
        s_lo = torch.cat([sol, zero])
        th_up = torch.cat([zero, th])
        th_lo = torch.cat([th, zero])
        rn = rexp + dt * (-s_up + s_lo) / vol
        rtn = rtexp + dt * (-th_up * s_up + th_lo * s_lo) / vol
        dint = 0.5 * (rn[:-1] + rn[1:])
        w_in = (2.0 * sol / G.area_v[1:L] - dint * wo) / rho_io
        w_new = torch.cat([so["w"][0:1], w_in, so["w"][L:L + 1]])
        tpn = rtn / rn - G.theta_bg
        epn = so["ep"] + vol * gam * (rtn - so["rt"])
        return {"rho": rn, "rt": rtn, "tp": tpn, "ep": epn, "w": w_new}

    def step(self, so, aux, first):
        """one step from the step-start state so (theta_v' rediagnosed); aux =
        (P, pvt, v2g) of the previous step or None; returns (state, aux)"""
        G, dt, iw = self.G, self.dt, self.iw
        L = G.nl
        P = self.pgrad(so)
        pgo_h = -P[1] if first else -aux[0][1]
        if first:
            pvt, v2g = self.advection(so)
        else:
            pvt, v2g = aux[1], aux[2]
        cur_hor, old_hor, cur_ver = 0.5 + iw, 1.0 - (0.5 + iw), 1.0 - iw

        def tend_w(P, pvt, v2g):
            t = -cur_ver * P[0] + pvt[0] - 0.5 * v2g[0]
            t = torch.cat([torch.zeros(1, G.nc, dtype=T0), t[1:L], torch.zeros(1, G.nc, dtype=T0)])
            return t

        tu0 = old_hor * pgo_h - cur_hor * P[1] + pvt[1] - 0.5 * v2g[1]
        tw0 = tend_w(P, pvt, v2g)
        u1 = so["u"] + dt * tu0
        sr, srt = self.scalar(so["rho"], so["rt"], u1)
        s1 = self.waves(so, so, sr, srt, tw0, 0)
        s1["u"] = u1
        pvt1, v2g1 = self.advection(s1)
        tu1 = 0.5 * tu0 + 0.5 * (old_hor * pgo_h - cur_hor * P[1] + pvt1[1] - 0.5 * v2g1[1])
        tw1 = 0.5 * tw0 + 0.5 * tend_w(P, pvt1, v2g1)
        u2 = so["u"] + dt * tu1
        sr, srt = self.scalar(s1["rho"], s1["rt"], u2)
        s2 = self.waves(so, s1, sr, srt, tw1, 1)
        s2["u"] = u2
        return s2, (P, pvt1, v2g1)

    def rediag(self, s):
        s = dict(s)
        s["tp"] = s["rt"] / s["rho"] - self.G.theta_bg
        return s

    def window(self, x0, n_steps, first=True, aux=None):
        s = self.rediag(x0)
        for n in range(n_steps):
            s2, aux = self.step(s, aux, first and n == 0)
            s = self.rediag(s2)
        return s2

    def sfc_pressure(self, s):
        G = self.G
        L = G.nl
        lapse = 0.0065
        t_low = (G.theta_bg[L - 1] + s["tp"][L - 1]) * (G.exner_bg[L - 1] + s["ep"][L - 1])
        p = s["rho"][L - 1] * R_D * t_low
        t_sfc = t_low + lapse * (G.z_scalar[L - 1] - G.zvec_v[L])
        ex = self.gm_low / (R_D * lapse)
        return p / torch.pow(1.0 - (t_sfc - t_low) / t_sfc, ex)


# ------------------------------------------------------------- host <-> tensors
def state_tensors(m, s):
    """a reference-layout State -> dict of 2-D tensors (dry)"""
    lay = m.layout
    nc, ne, L = lay.nc, lay.ne, lay.nl
    vpl = nc + ne
    t = lambda a: torch.tensor(np.ascontiguousarray(a), dtype=T0)
    wind = np.asarray(s["wind"])
    return {"rho": t(np.asarray(s["rho"]).reshape(L, nc)), "rt": t(np.asarray(s["rhotheta_v"]).reshape(L, nc)),
            "tp": t(np.asarray(s["theta_v_pert"]).reshape(L, nc)), "ep": t(np.asarray(s["exner_pert"]).reshape(L, nc)),
            "w": t(np.stack([wind[k * vpl:k * vpl + nc] for k in range(L + 1)])),
            "u": t(np.stack([wind[nc + l * vpl:(l + 1) * vpl] for l in range(L)]))}


def tensors_to_state(m, d, out):
    """dict of 2-D arrays -> reference-layout State arrays of out"""
    lay = m.layout
    nc, ne, L = lay.nc, lay.ne, lay.nl
    vpl = nc + ne
    a = lambda x: x.detach().numpy() if isinstance(x, torch.Tensor) else np.asarray(x)
    out["rho"][:] = a(d["rho"]).ravel()
    out["rhotheta_v"][:] = a(d["rt"]).ravel()
    out["theta_v_pert"][:] = a(d["tp"]).ravel() if d.get("tp") is not None else 0.0
    out["exner_pert"][:] = a(d["ep"]).ravel()
    wind = np.zeros(lay.n_vectors)
    for k in range(L + 1):
        wind[k * vpl:k * vpl + nc] = a(d["w"])[k]
    for l in range(L):
        wind[nc + l * vpl:(l + 1) * vpl] = a(d["u"])[l]
    out["wind"][:] = wind


def fv_bounds(m):
    """flux_density at levels 0 and L (never written by the step)"""
    lay = m.layout
    fl = np.asarray(m.diagnostics["flux_density"])
    vpl = lay.nc + lay.ne
    return torch.tensor(np.stack([fl[0:lay.nc], fl[lay.nl * vpl:lay.nl * vpl + lay.nc]]), dtype=T0)


def make_step(m, dt):
    st = DryStep(m, dt)
    st.fv_bounds = fv_bounds(m)
    lay = m.layout
    vpl = lay.nc + lay.ne
    gm = np.asarray(m.grid["gravity_m"])
    st.gm_low = torch.tensor(gm[(lay.nl - 1) * vpl:(lay.nl - 1) * vpl + lay.nc], dtype=T0)
    return st
