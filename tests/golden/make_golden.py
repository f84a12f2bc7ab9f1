"""Generate the closed-form known-answer fixtures in this directory.

The reference (zeshunzong/reduced_mpm_stress_training) ships no tests or
golden vectors, and its Warp solver cannot run here, so these fixtures are
analytic: each value is computed with plain ``math`` from the formulas of
the reference, written out independently of the oracle's code.

  kat_return_map.json  return mapping + Kirchhoff stress of DIAGONAL F_trial
                       (SVD factors are signed permutations, so the result is
                       closed-form): sand (engine_stress/mpm_utils.py:87-112,
                       :45-52), metal (:59-84, :36-43), jelly (:29-34)
  kat_p2g.json         one particle's P2G contributions to its 27 nodes
                       (engine_stress/mpm_utils.py:190-227)
  kat_reduced_p2g.json one particle's reduced-substep P2G with a diagonal F_disp
                       (engine_stress/mpm_utils.py:353-402, stresses :29-34, :45-52)
  kat_decoder.json     the stress decoder NetDec with hand-set weights on four rows,
                       ELU and SIREN (offline_training_xhat_and_stress_and_mu/
                       CROMnet_secondary.py:203-301, 447-525)

Run:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import json
import math
import os

HERE = os.path.dirname(os.path.abspath(__file__))


def lame(E, nu):
    return E / 2.0 / (1.0 + nu), E * nu / (1.0 + nu) / (1.0 - 2.0 * nu)


def alpha(phi):
    s = math.sin(phi / 180.0 * 3.14159265)
    return math.sqrt(2.0 / 3.0) * 2.0 * s / (3.0 - s)


def sand(eps, mu, lam, al):
    tr = sum(eps)
    eh = [e - tr / 3 for e in eps]
    ehn = math.sqrt(sum(x * x for x in eh))
    dg = ehn + (3 * lam + 2 * mu) / (2 * mu) * tr * al
    if dg <= 0:
        H, case = list(eps), "elastic"
    elif tr > 0:
        H, case = [0.0, 0.0, 0.0], "tension"
    else:
        H, case = [eps[i] - eh[i] * (dg / ehn) for i in range(3)], "shear"
    F = [math.exp(h) for h in H]
    ls = sum(H)
    tau = [2 * mu * H[i] + lam * ls for i in range(3)]
    return F, tau, case


def metal(eps_in, mu, lam, ys):
    sig = [max(math.exp(e), 0.01) for e in eps_in]
    eps = [math.log(s) for s in sig]
    es = sum(eps)
    t = [2 * mu * e + lam * es for e in eps]
    st = sum(t)
    cond = math.sqrt(sum((ti - st / 3) ** 2 for ti in t))
    if cond > ys:
        mean = es / 3
        eh = [e - mean for e in eps]
        n = math.sqrt(sum(x * x for x in eh)) + 1e-6
        dg = n - ys / (2 * mu)
        eps2 = [eps[i] - (dg / n) * eh[i] for i in range(3)]
        F = [math.exp(e) for e in eps2]
        case = "plastic"
    else:
        F = [math.exp(e) for e in eps_in]
        case = "elastic"
    l = [math.log(max(f, 0.01)) for f in F]
    ls = sum(l)
    tau = [2 * mu * li + lam * ls for li in l]
    return F, tau, case


def jelly(eps, mu, lam):
    F = [math.exp(e) for e in eps]
    J = F[0] * F[1] * F[2]
    tau = [2 * mu * (F[i] - 1.0) * F[i] + lam * J * (J - 1.0) for i in range(3)]
    return F, tau, "elastic"


def diag9(d):
    return [d[0], 0.0, 0.0, 0.0, d[1], 0.0, 0.0, 0.0, d[2]]


def make_return_map():
    cases = []
    strains = [
        [0.0, 0.0, 0.0], [0.01, -0.02, 0.005], [-0.01, -0.01, -0.01], [0.02, 0.02, 0.02],
        [-0.05, 0.01, 0.0], [-0.2, -0.05, 0.03], [0.1, -0.3, -0.1], [-0.001, 0.0005, 0.0002],
        [0.05, -0.02, -0.04], [-0.15, -0.15, 0.1],
    ]
    for E, nu, phi in [(2e5, 0.3, 30.0), (3e5, 0.3, 35.0)]:
        mu, lam = lame(E, nu)
        al = alpha(phi)
        for eps in strains:
            F, tau, case = sand(eps, mu, lam, al)
            cases.append(dict(material="sand", E=E, nu=nu, friction_angle=phi, yield_stress=0.0,
                              F_trial=diag9([math.exp(e) for e in eps]), F=diag9(F),
                              stress=diag9(tau), case=case))
    mu, lam = lame(1e7, 0.3)
    for eps in strains:
        F, tau, case = metal(eps, mu, lam, 1e5)
        cases.append(dict(material="metal", E=1e7, nu=0.3, friction_angle=30.0, yield_stress=1e5,
                          F_trial=diag9([math.exp(e) for e in eps]), F=diag9(F),
                          stress=diag9(tau), case=case))
    mu, lam = lame(2e5, 0.3)
    for eps in strains:
        F, tau, case = jelly(eps, mu, lam)
        cases.append(dict(material="jelly", E=2e5, nu=0.3, friction_angle=30.0, yield_stress=0.0,
                          F_trial=diag9([math.exp(e) for e in eps]), F=diag9(F),
                          stress=diag9(tau), case=case))
    return cases


def make_p2g():
    """One particle, n_grid 16, dx 1/16: per-node (mass, momentum) contributions."""
    n, lim = 16, 1.0
    dx = lim / n
    inv_dx = n / lim
    x = [0.4137, 0.5261, 0.3319]
    v = [0.3, -0.2, 0.1]
    Cm = [0.5, -0.1, 0.2, 0.05, -0.3, 0.1, 0.0, 0.2, -0.4]
    tau = [1200.0, 300.0, -150.0, 300.0, -800.0, 50.0, -150.0, 50.0, 400.0]
    m, vol, dt = 2.0e-4, 1.0e-7, 1e-4
    base, fx = [], []
    for d in range(3):
        gp = x[d] * inv_dx
        b = int(gp - 0.5)
        base.append(b)
        fx.append(gp - b)
    w = [[0.5 * (1.5 - f) ** 2, 0.75 - (f - 1.0) ** 2, 0.5 * (f - 0.5) ** 2] for f in fx]
    dw = [[f - 1.5, -2.0 * (f - 1.0), f - 0.5] for f in fx]
    nodes = []
    for i in range(3):
        for j in range(3):
            for k in range(3):
                wt = w[0][i] * w[1][j] * w[2][k]
                gw = [dw[0][i] * w[1][j] * w[2][k] * inv_dx, w[0][i] * dw[1][j] * w[2][k] * inv_dx,
                      w[0][i] * w[1][j] * dw[2][k] * inv_dx]
                dpos = [(i - fx[0]) * dx, (j - fx[1]) * dx, (k - fx[2]) * dx]
                mom = []
                for r in range(3):
                    cd = sum(Cm[3 * r + c] * dpos[c] for c in range(3))
                    f = sum(-vol * tau[3 * r + c] * gw[c] for c in range(3))
                    mom.append(wt * m * (v[r] + cd) + dt * f)
                nodes.append(dict(index=[base[0] + i, base[1] + j, base[2] + k], mass=wt * m,
                                  momentum=mom))
    return dict(n_grid=n, grid_lim=lim, x=x, v=v, C=Cm, stress=tau, mass=m, vol=vol, dt=dt,
                nodes=nodes)


def make_reduced_p2g():
    """One particle through p2g_sample_all (engine_stress/mpm_utils.py:353-402) with a
    diagonal F_disp, so F = I + F_disp is its own SVD and the stress is closed-form:
    FCR for jelly and metal (:29-34, R = I, J = s0 s1 s2), Drucker-Prager for sand
    (:45-52, U diag(c) V^T F^T = diag(c_i s_i)).  No affine term; the force uses the
    volume m / density.  Per-node (mass, momentum) after the three adds."""
    n, lim = 16, 1.0
    inv_dx = n / lim
    x = [0.4137, 0.5261, 0.3319]
    v = [0.3, -0.2, 0.1]
    fdisp = [0.02, -0.03, 0.01]
    m, rho, dt = 2.0e-4, 2000.0, 1e-4
    base, fx = [], []
    for d in range(3):
        gp = x[d] * inv_dx
        b = int(gp - 0.5)
        base.append(b)
        fx.append(gp - b)
    w = [[0.5 * (1.5 - f) ** 2, 0.75 - (f - 1.0) ** 2, 0.5 * (f - 0.5) ** 2] for f in fx]
    dw = [[f - 1.5, -2.0 * (f - 1.0), f - 0.5] for f in fx]
    sig = [1.0 + f for f in fdisp]
    out = []
    for material, E, nu in (("jelly", 2e5, 0.3), ("metal", 1e7, 0.3), ("sand", 2e5, 0.3)):
        mu, lam = lame(E, nu)
        if material == "sand":
            ls = sum(math.log(s) for s in sig)
            tau = [(2 * mu * math.log(s) + lam * ls) / s * s for s in sig]
        else:
            J = sig[0] * sig[1] * sig[2]
            tau = [2 * mu * (s - 1.0) * s + lam * J * (J - 1.0) for s in sig]
        nodes = []
        for i in range(3):
            for j in range(3):
                for k in range(3):
                    wt = w[0][i] * w[1][j] * w[2][k]
                    gw = [dw[0][i] * w[1][j] * w[2][k] * inv_dx, w[0][i] * dw[1][j] * w[2][k] * inv_dx,
                          w[0][i] * w[1][j] * dw[2][k] * inv_dx]
                    mom = [wt * m * v[r] + dt * (-(m / rho) * tau[r] * gw[r]) for r in range(3)]
                    nodes.append(dict(index=[base[0] + i, base[1] + j, base[2] + k], mass=wt * m, momentum=mom))
        out.append(dict(material=material, E=E, nu=nu, n_grid=n, grid_lim=lim, x=x, v=v, F_disp=diag9(fdisp),
                        mass=m, density=rho, dt=dt, stress=diag9(tau), nodes=nodes))
    return out


def make_decoder():
    """NetDec (offline_training_xhat_and_stress_and_mu/CROMnet_secondary.py:203-301) with
    small hand-set weights, evaluated with plain math: Prepare (standardise, or clip to
    [-1, 1] with SIREN; :507-525), five Linear + activation (ELU / sin(30 x); :447-463),
    Linear to 6, mean_q + q * std_q (:476-477).  label 2, mu 1, hidden 3."""
    lbl, mu_dim, h = 2, 1, 3
    n_in = lbl + 3 + mu_dim

    def lin(W, b, x):
        return [b[j] + sum(W[j][k] * x[k] for k in range(len(x))) for j in range(len(W))]

    sd = {"dec0.weight": [[0.1 * (j + 1) - 0.05 * k for k in range(n_in)] for j in range(h)],
          "dec0.bias": [0.01 * j for j in range(h)]}
    for l, name in enumerate(("dec1", "dec2", "dec3", "dec4")):
        sd[name + ".weight"] = [[((j + k + l) % 3 - 1) * 0.5 for k in range(h)] for j in range(h)]
        sd[name + ".bias"] = [-0.1 + 0.05 * l + 0.02 * j for j in range(h)]
    sd["enc.weight"] = [[0.2 * (c - k) for k in range(h)] for c in range(6)]
    sd["enc.bias"] = [float(c) for c in range(6)]
    sd["invStandardizeQ.mean_q_torch"] = [1.0, 2.0, 3.0, 4.0, 5.0, 6.0]
    sd["invStandardizeQ.std_q_torch"] = [2.0, 0.5, 1.0, 3.0, 0.25, 1.5]
    rows = [[0.3, -1.2, 0.45, 0.52, 0.31, 30.0], [-0.7, 0.1, 0.61, 0.38, 0.75, 25.0],
            [1.5, 0.4, 0.40, 0.50, 0.10, 35.0], [0.0, 0.0, 0.55, 0.45, 0.60, 20.0]]
    out = []
    for siren in (False, True):
        d = dict(sd)
        if siren:
            d["prepare.min_x_torch"], d["prepare.max_x_torch"] = [0.35, 0.35, 0.05], [0.65, 0.65, 0.85]
        else:
            d["prepare.mean_x_torch"], d["prepare.std_x_torch"] = [0.5, 0.5, 0.45], [0.25, 0.5, 1.0]
        q_all = []
        for r in rows:
            x = list(r)
            for c in range(3):
                if siren:
                    lo, hi = d["prepare.min_x_torch"][c], d["prepare.max_x_torch"][c]
                    x[lbl + c] = 2 * (r[lbl + c] - lo) / (hi - lo) - 1
                else:
                    x[lbl + c] = (r[lbl + c] - d["prepare.mean_x_torch"][c]) / d["prepare.std_x_torch"][c]

            def act(z):
                return math.sin(30.0 * z) if siren else (z if z > 0 else math.expm1(z))

            y = [act(z) for z in lin(d["dec0.weight"], d["dec0.bias"], x)]
            for name in ("dec1", "dec2", "dec3", "dec4"):
                y = [act(z) for z in lin(d[name + ".weight"], d[name + ".bias"], y)]
            q = lin(d["enc.weight"], d["enc.bias"], y)
            q_all.append([d["invStandardizeQ.mean_q_torch"][c] + q[c] * d["invStandardizeQ.std_q_torch"][c]
                          for c in range(6)])
        out.append(dict(siren=siren, omega_0=30.0, label_dim=lbl, mu_dim=mu_dim, hidden=h, state_dict=d,
                        rows=rows, q=q_all))
    return out


if __name__ == "__main__":
    with open(os.path.join(HERE, "kat_decoder.json"), "w") as f:
        json.dump(make_decoder(), f, indent=1)
    with open(os.path.join(HERE, "kat_reduced_p2g.json"), "w") as f:
        json.dump(make_reduced_p2g(), f, indent=1)
    with open(os.path.join(HERE, "kat_return_map.json"), "w") as f:
        json.dump(make_return_map(), f, indent=1)
    with open(os.path.join(HERE, "kat_p2g.json"), "w") as f:
        json.dump(make_p2g(), f, indent=1)
    print("wrote kat_return_map.json, kat_p2g.json, kat_reduced_p2g.json, kat_decoder.json")
