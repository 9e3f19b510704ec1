"""Synthetic blastwave histories: the per-step scalar records that the
reference's blastwave driver would hand to the comoving-radiation step.

The reference produces these from its ODE driver (src/model_evolve.h,
src/blastwave/) which is not part of this package. Here each jet layer follows
a simple adiabatic thin-shell model (swept-up mass m, Lorentz factor Gamma with
dGamma/dm = -(Gamma^2 - 1)/(M0 + 2 Gamma m), iso-equivalent radius from m),
sampled on the reference's burster-time grid; a reverse shock exists until the
ejecta are crossed. The shock scalars (B, gamma_min, gamma_max, gamma_c,
accel_frac, n') come from the library's restatement of
computeEleSpectrumLimits (microphysics_base.h:642-966), called exactly as the
driver calls it (blastwave_radiation.h:976-1107).

The value ranges (Lorentz factors, densities, cooling regimes, substep
counts from 1 to max_substeps, the gamma_min <= 2 analytic fallback late on)
follow the reference's configurations; the exact dynamics do not matter for the
comoving step, whose parity is checked on identical records.

driver_records / DriverRun build the same records from the dynamics the
reference's own program saved (a recorded run), exactly as its driver passes
them to the step, so that the step mix is the reference's own.
"""
from dataclasses import dataclass, field

import numpy as np

from . import abi

C_LIGHT = 2.99792458e10
M_P = 1.6726e-24


@dataclass
class Shock:
    """Microphysics parameters of one shock (the *_fs / *_rs parfile keys)."""
    eps_e: float = 0.1
    eps_b: float = 1e-3
    p: float = 2.2
    ssc: bool = False
    ssa: bool = False
    max_substeps: int = 1000
    ele_method: int = abi.PBAG_ELE_NUMERIC
    syn_method: int = abi.PBAG_SYN_CSYN
    adi: bool = True
    # computeEleSpectrumLimits' methods (pbag_limits_opts codes; the
    # reference's parfile defaults are useNumeric / useTcomov / useB /
    # useU_b / use_Sironi = 1, 1, 0, 0, 3)
    method_gamma_min: int = 0
    method_gamma_c: int = 0
    method_gamma_max: int = 0
    method_B: int = 0
    method_nonrel: int = 0


@dataclass
class JetConfig:
    """One jet: structure, energetics, ISM, grids and time grid."""
    struct: str = "tophat"            # "tophat" or "gaussian"
    E_iso: float = 1e52               # core isotropic energy [erg]
    Gamma0: float = 300.0             # core initial Lorentz factor
    theta_c: float = 0.1              # core half-opening angle [rad]
    theta_w: float = 0.1              # wing angle [rad] (gaussian)
    n_ism: float = 1e-2               # ISM density [cm^-3]
    nlayers: int = 1
    fs: Shock = field(default_factory=Shock)
    rs: Shock = None                  # None: forward shock only
    ngam: int = 151
    gam1: float = 1.0
    gam2: float = 1e8
    nfreq: int = 96
    freq1: float = 1e8
    freq2: float = 1e29
    ntb: int = 1000
    tb1: float = 3e2
    tb2: float = 1e14

    def grid(self):
        return abi.GridDesc(self.ngam, self.nfreq, self.gam1, self.gam2, self.freq1, self.freq2)


def config_tophat_fs():
    """One top-hat layer, forward shock only, synchrotron only (the
    reference's CPU-runnable case): E_iso=1e52, Gamma0=300, theta_c=0.1,
    n=1e-2, eps_e=0.1, eps_b=1e-3, p=2.2, 151 gamma x 96 nu, ntb=1000."""
    return JetConfig()


def config_gaussian_ssc():
    """The 21-layer Gaussian jet with forward and reverse shocks, synchrotron +
    SSC (+SSA): Eiso_c=10^54.1, Gamma0c=300, theta_c=3.5 deg, theta_w=25 deg,
    n=10^-1.6, eps_e=10^-3.42, eps_b=10^-4.02, p=2.1, 201 gamma in [1,1e9],
    128 nu in [1e8,1e29], ntb=1000."""
    sh = dict(eps_e=10 ** -3.42, eps_b=10 ** -4.02, p=2.1, ssc=True, ssa=True)
    return JetConfig(struct="gaussian", E_iso=10 ** 54.1, Gamma0=300.0,
                     theta_c=np.deg2rad(3.5), theta_w=np.deg2rad(25.0),
                     n_ism=10 ** -1.6, nlayers=21, fs=Shock(**sh), rs=Shock(**sh),
                     ngam=201, gam1=1.0, gam2=1e9, nfreq=128)


def layer_table(cfg):
    """(theta_lo, theta_hi, E_iso, Gamma0) per layer."""
    tw = cfg.theta_c if cfg.struct == "tophat" else cfg.theta_w
    edges = np.linspace(0.0, tw, cfg.nlayers + 1)
    mid = 0.5 * (edges[1:] + edges[:-1])
    if cfg.struct == "tophat":
        E = np.full(cfg.nlayers, cfg.E_iso)
        G0 = np.full(cfg.nlayers, cfg.Gamma0)
    else:
        w = np.exp(-0.5 * (mid / cfg.theta_c) ** 2)
        E = cfg.E_iso * w
        G0 = 1.0 + (cfg.Gamma0 - 1.0) * w
    G0 = np.maximum(G0, 1.5)
    return edges[:-1], edges[1:], E, G0


def _rk4(f, y, x0, x1, n):
    h = (x1 - x0) / n
    x = x0
    out = [y.copy()]
    for _ in range(n):
        k1 = f(x, y)
        k2 = f(x + h / 2, y + h / 2 * k1)
        k3 = f(x + h / 2, y + h / 2 * k2)
        k4 = f(x + h, y + h * k3)
        y = y + h / 6 * (k1 + 2 * k2 + 2 * k3 + k4)
        x += h
        out.append(y.copy())
    return np.array(out)


def layer_dynamics(E_iso, Gamma0, n_ism, tb, omega, nsamp=4000):
    """Thin-shell dynamics of one layer sampled at burster times tb.

    Integrates in x = ln m_iso the variables (u = ln(Gamma-1), t_b, t_comov,
    t_obs) with R = (3 m / 4 pi rho)^(1/3); returns arrays on tb."""
    rho = n_ism * M_P
    M0 = E_iso / ((Gamma0 - 1.0) * C_LIGHT ** 2)
    beta0 = np.sqrt(1 - 1 / Gamma0 ** 2)
    # start well inside the coasting phase, at the radius reached by tb[0]/10
    R0 = beta0 * C_LIGHT * tb[0] * 0.1
    m0 = 4 / 3 * np.pi * R0 ** 3 * rho
    m1 = max(1e6 * M0 * Gamma0, m0 * 1e40)

    def rhs(x, y):
        m = np.exp(x)
        gm1 = max(np.exp(y[0]), 1e-300)      # Gamma - 1, kept apart from 1 for precision
        G = 1.0 + gm1
        # dGamma/dm / (Gamma - 1) = -(Gamma + 1)/(M0 + 2 Gamma m)
        dudm = -(G + 1.0) / (M0 + 2.0 * G * m)
        R = (3 * m / (4 * np.pi * rho)) ** (1 / 3)
        dRdx = R / 3.0                       # dR/dln m
        beta = np.sqrt(gm1 * (2.0 + gm1)) / G
        return np.array([dudm * m,
                         dRdx / (beta * C_LIGHT),
                         dRdx / (beta * G * C_LIGHT),
                         dRdx * (1 - beta) / (beta * C_LIGHT)])

    y0 = np.array([np.log(Gamma0 - 1.0), R0 / (beta0 * C_LIGHT),
                   R0 / (beta0 * Gamma0 * C_LIGHT), R0 * (1 - beta0) / (beta0 * C_LIGHT)])
    xs = np.linspace(np.log(m0), np.log(m1), nsamp + 1)
    ys = _rk4(rhs, y0, xs[0], xs[-1], nsamp)
    t_b = ys[:, 1]
    lt = np.log(t_b)
    lq = np.log(tb)
    x = np.interp(lq, lt, xs)
    u = np.interp(lq, lt, ys[:, 0])
    tcom = np.exp(np.interp(lq, lt, np.log(ys[:, 2])))
    tobs = np.exp(np.interp(lq, lt, np.log(ys[:, 3])))
    m_iso = np.exp(x)
    gm1 = np.maximum(np.exp(u), 1e-300)
    G = 1.0 + gm1
    beta = np.sqrt(gm1 * (2.0 + gm1)) / G
    R = (3 * m_iso / (4 * np.pi * rho)) ** (1 / 3)
    frac = omega / (4 * np.pi)
    return dict(Gamma=G, beta=beta, R=R, m=m_iso * frac, m_iso=m_iso, tcomov=tcom,
                t_obs=tobs, M0=M0 * frac, M0_iso=M0, Gamma0=Gamma0, beta0=beta0, rho=rho)


def fs_state(d):
    """Forward-shock downstream quantities (iso-equivalent thin shell)."""
    G = d["Gamma"]
    gad = (4.0 + 1.0 / G) / 3.0                               # adiabatic index
    rho2 = (gad * G + 1.0) / (gad - 1.0) * d["rho"]           # comoving density
    m2 = d["m"]
    u_p = (G - 1.0) * rho2 * C_LIGHT ** 2                     # comoving energy density
    thick = d["m_iso"] / (4 * np.pi * d["R"] ** 2 * G * rho2)  # lab-frame thickness
    return dict(Gamma=G, GammaSh=G, rho2=rho2, m2=m2, u_p=u_p, thick=thick,
                dr=thick * G, valid=np.ones_like(G, dtype=bool))


def rs_state(d, shell_width=3e12):
    """Reverse shock in the ejecta, active until the shell is crossed at the
    deceleration radius, then until it has expanded a further factor 3."""
    G, G0, b0 = d["Gamma"], d["Gamma0"], d["beta0"]
    beta = d["beta"]
    G43 = np.maximum(G0 * G * (1.0 - b0 * beta), 1.0 + 1e-9)
    Rx = (3 * d["M0_iso"] / G0 / (4 * np.pi * d["rho"])) ** (1 / 3)  # m = M0/Gamma0
    R = d["R"]
    xfrac = np.minimum(1.0, (R / Rx) ** 1.5)
    m3 = d["M0"] * np.maximum(xfrac, 1e-6)
    rho_ej = d["M0_iso"] / (4 * np.pi * R ** 2 * shell_width * G0)
    gad = (4.0 + 1.0 / G43) / 3.0
    rho3 = (gad * G43 + 1.0) / (gad - 1.0) * rho_ej
    u_p3 = (G43 - 1.0) * rho3 * C_LIGHT ** 2
    thick = d["M0_iso"] * np.maximum(xfrac, 1e-6) / (4 * np.pi * R ** 2 * G * rho3)
    valid = R < 3.0 * Rx
    return dict(Gamma=G, GammaSh=G43, rho2=rho3, m2=m3, u_p=u_p3, thick=thick,
                dr=thick * G43, valid=valid)


def limits_opts(sh):
    o = abi.LimitsOpts()
    o.p, o.eps_e, o.eps_b, o.eps_t = sh.p, sh.eps_e, sh.eps_b, 0.0
    o.beta_min, o.mu, o.mu_e = 1e-5, 0.62, 1.18
    o.method_B = sh.method_B
    o.method_gamma_min = sh.method_gamma_min
    o.method_gamma_c = sh.method_gamma_c
    o.method_gamma_max = sh.method_gamma_max
    o.method_nonrel = sh.method_nonrel
    o.ele_analytic = 0
    return o


def shock_records(lib, st, d, sh, gam, tb):
    """Step records of one shock: computeEleSpectrumLimits on every step, then
    the arguments of init/evolve exactly as blastwave_radiation.h:1109-1182."""
    n = len(tb)
    ss = np.zeros(n, dtype=abi.SHOCK_STATE_DTYPE)
    ss["e_prime"] = st["u_p"]
    ss["Gamma"] = st["Gamma"]
    ss["GammaSh"] = st["GammaSh"]
    ss["t_e"] = d["t_obs"]
    ss["t_b"] = tb
    ss["tcomov"] = d["tcomov"]
    ss["n_prime"] = st["rho2"] / M_P
    ss["n_protons"] = st["m2"] / M_P
    lim = lib.shock_limits(limits_opts(sh), gam, ss)
    recs = np.zeros(n, dtype=abi.STEP_DTYPE)
    valid = st["valid"] & (lim["valid"] == 1) & (st["u_p"] > 0) & (st["rho2"] > 0)
    recs["mode"] = np.where(valid, abi.PBAG_EVOLVE, abi.PBAG_SKIP)
    first = np.argmax(valid) if valid.any() else n
    if first < n:
        recs["mode"][first] = abi.PBAG_INIT
    prev = lambda a: np.concatenate([a[:1], a[:-1]])
    recs["tc"], recs["tc_p1"] = prev(d["tcomov"]), d["tcomov"]
    recs["m"], recs["m_p1"] = prev(st["m2"]), st["m2"]
    recs["rho"], recs["rho_p1"] = prev(st["rho2"]), st["rho2"]
    recs["u_p"], recs["u_p_p1"] = prev(st["u_p"]), st["u_p"]
    dr = st["dr"]
    recs["dr"], recs["dr_p1"] = prev(dr), dr
    # the first valid step passes the current thickness to initializeElectronDistribution
    if first < n:
        recs["dr"][first] = st["thick"][first]
    for k in ("B", "gamma_min", "gamma_max", "gamma_c", "accel_frac"):
        recs[k] = lim[k]
    recs["n_prime"] = ss["n_prime"]
    return recs


def shock_params(sh):
    p = np.zeros(1, dtype=abi.SHOCK_PARAMS_DTYPE)
    p["p"], p["eps_e"], p["max_substeps"] = sh.p, sh.eps_e, sh.max_substeps
    p["ele_method"], p["syn_method"] = sh.ele_method, sh.syn_method
    p["ssa_on"], p["ssc_on"], p["adi_on"], p["pp_on"] = int(sh.ssa), int(sh.ssc), int(sh.adi), 0
    return p[0]


def layer_dynamics_many(E_iso, Gamma0, n_ism, tb, omega, nsamp=4000):
    """layer_dynamics for every layer of a jet at once (the RK4 steps of all
    layers advance together, elementwise the same arithmetic)."""
    E_iso, Gamma0, omega = (np.asarray(a, dtype=np.float64) for a in (E_iso, Gamma0, omega))
    L = len(E_iso)
    rho = n_ism * M_P
    M0 = E_iso / ((Gamma0 - 1.0) * C_LIGHT ** 2)
    beta0 = np.sqrt(1 - 1 / Gamma0 ** 2)
    R0 = beta0 * C_LIGHT * tb[0] * 0.1
    m0 = 4 / 3 * np.pi * R0 ** 3 * rho
    m1 = np.maximum(1e6 * M0 * Gamma0, m0 * 1e40)

    def rhs(x, y):
        m = np.exp(x)
        gm1 = np.maximum(np.exp(y[0]), 1e-300)
        G = 1.0 + gm1
        dudm = -(G + 1.0) / (M0 + 2.0 * G * m)
        R = (3 * m / (4 * np.pi * rho)) ** (1 / 3)
        dRdx = R / 3.0
        beta = np.sqrt(gm1 * (2.0 + gm1)) / G
        return np.stack([dudm * m, dRdx / (beta * C_LIGHT), dRdx / (beta * G * C_LIGHT),
                         dRdx * (1 - beta) / (beta * C_LIGHT)])

    y = np.stack([np.log(Gamma0 - 1.0), R0 / (beta0 * C_LIGHT), R0 / (beta0 * Gamma0 * C_LIGHT),
                  R0 * (1 - beta0) / (beta0 * C_LIGHT)])
    x0, x1 = np.log(m0), np.log(m1)
    h = (x1 - x0) / nsamp
    x = x0.copy()
    ys = np.empty((nsamp + 1, 4, L))
    xs = np.empty((nsamp + 1, L))
    ys[0], xs[0] = y, x
    for i in range(nsamp):
        k1 = rhs(x, y)
        k2 = rhs(x + h / 2, y + h / 2 * k1)
        k3 = rhs(x + h / 2, y + h / 2 * k2)
        k4 = rhs(x + h, y + h * k3)
        y = y + h / 6 * (k1 + 2 * k2 + 2 * k3 + k4)
        x = x + h
        ys[i + 1], xs[i + 1] = y, x
    out = []
    lq = np.log(tb)
    for l in range(L):
        lt = np.log(ys[:, 1, l])
        xl = np.interp(lq, lt, xs[:, l])
        u = np.interp(lq, lt, ys[:, 0, l])
        tcom = np.exp(np.interp(lq, lt, np.log(ys[:, 2, l])))
        tobs = np.exp(np.interp(lq, lt, np.log(ys[:, 3, l])))
        m_iso = np.exp(xl)
        gm1 = np.maximum(np.exp(u), 1e-300)
        G = 1.0 + gm1
        beta = np.sqrt(gm1 * (2.0 + gm1)) / G
        R = (3 * m_iso / (4 * np.pi * rho)) ** (1 / 3)
        frac = omega[l] / (4 * np.pi)
        out.append(dict(Gamma=G, beta=beta, R=R, m=m_iso * frac, m_iso=m_iso, tcomov=tcom, t_obs=tobs,
                        M0=M0[l] * frac, M0_iso=M0[l], Gamma0=Gamma0[l], beta0=beta0[l], rho=rho))
    return out


def make_batch(lib, cfg, nsteps=None):
    """Records for every blastwave of one jet: (recs, offsets, params, grid).

    Blastwaves are ordered layer by layer, forward shock then reverse shock.
    nsteps truncates every history to its first nsteps burster times."""
    tb = np.logspace(np.log10(cfg.tb1), np.log10(cfg.tb2), cfg.ntb)
    if nsteps is not None:
        tb = tb[:nsteps]
    grid = cfg.grid()
    gam, _ = lib.grids(grid)
    lo, hi, E, G0 = layer_table(cfg)
    omega = 2 * np.pi * (np.cos(lo) - np.cos(hi)) * 2  # both hemispheres
    dyn = layer_dynamics_many(E, G0, cfg.n_ism, tb, omega)
    recs, params = [], []
    for il in range(cfg.nlayers):
        d = dyn[il]
        recs.append(shock_records(lib, fs_state(d), d, cfg.fs, gam, tb))
        params.append(shock_params(cfg.fs))
        if cfg.rs is not None:
            recs.append(shock_records(lib, rs_state(d), d, cfg.rs, gam, tb))
            params.append(shock_params(cfg.rs))
    offsets = np.zeros(len(recs) + 1, dtype=np.int64)
    offsets[1:] = np.cumsum([len(r) for r in recs])
    return np.concatenate(recs), offsets, np.array(params, dtype=abi.SHOCK_PARAMS_DTYPE), grid


def driver_records(lib, dyn, shocks, gam, beta_min=1e-5):
    """Step records of every blastwave of a jet from the dynamics its ODE
    driver saved, following the driver's in-situ calls
    (blastwave_radiation.h:881-1198): at every time index `it` the blastwave
    is valid (isBlastWaveValidForElectronCalc, :881-959: R >= 1, beta >=
    beta_min, U_p > 0, rho2 > 0); the forward shock's limits come from
    updateSockProperties(U_p, Gamma, GammaFsh, tt, tburst, tcomov, rho2/m_p,
    M2/m_p) (:1047-1066), its step is initializeElectronDistribution(tcomov,
    M2, rho2, U_p, thickness) on the first valid index and
    evaluateElectronDistributionNumericMixed with the comoving thickness
    thickness * GammaFsh at it-1 and it afterwards (:1147-1182); the reverse
    shock, where considerReverseShock holds (:961-974: it > 0, the RS
    thickness at it-1, GammaRsh and U_p3 positive), the same with U_p3,
    GammaRsh, rho3, M3, thichness_rs - its comoving thickness at `it` is
    multiplied by GammaRsh at it-1, as the driver does (:1125-1129).

    dyn: one dict per layer of the saved histories by their names
    (BW::VARNAMES); shocks: (forward, reverse-or-None) Shock options.
    Returns (recs, offsets, params); blastwaves layer by layer, forward shock
    then reverse shock."""
    recs, params = [], []
    mp = M_P
    for d in dyn:
        n = len(d["tburst"])
        valid = (d["R"] >= 1) & (d["beta"] >= beta_min) & (d["U_p"] > 0) & (d["rho2"] > 0)
        for is_rs, sh in ((False, shocks[0]), (True, shocks[1])):
            if sh is None:
                continue
            if is_rs and "U_p3" not in d:
                # a layer whose Gamma0 is below min_Gamma0_for_rs runs no
                # reverse shock (blastwave_base.h:449-453) and saves no
                # reverse-shock quantities: its blastwave is all skips
                r = np.zeros(n, dtype=abi.STEP_DTYPE)
                r["mode"] = abi.PBAG_SKIP
                recs.append(r)
                params.append(shock_params(sh))
                continue
            if is_rs:
                up, gsh, rho, m, th = d["U_p3"], d["GammaRsh"], d["rho3"], d["M3"], d["thichness_rs"]
                prev_th = np.concatenate([[0.0], th[:-1]])
                ok = valid & (np.arange(n) > 0) & (prev_th > 0) & (gsh > 0) & (up > 0)
            else:
                up, gsh, rho, m, th = d["U_p"], d["GammaFsh"], d["rho2"], d["M2"], d["thickness"]
                ok = valid.copy()
            ss = np.zeros(n, dtype=abi.SHOCK_STATE_DTYPE)
            ss["e_prime"], ss["Gamma"], ss["GammaSh"] = up, d["Gamma"], gsh
            ss["t_e"], ss["t_b"], ss["tcomov"] = d["tt"], d["tburst"], d["tcomov"]
            ss["n_prime"], ss["n_protons"] = rho / mp, m / mp
            # the driver updates the shock only at the steps it runs, in order
            lim = np.zeros(n, dtype=abi.LIMITS_DTYPE)
            if ok.any():
                lim[ok] = lib.shock_limits(limits_opts(sh), gam, ss[ok])
            r = np.zeros(n, dtype=abi.STEP_DTYPE)
            r["mode"] = np.where(ok, abi.PBAG_EVOLVE, abi.PBAG_SKIP)
            first = int(np.argmax(ok)) if ok.any() else n
            if first < n:
                r["mode"][first] = abi.PBAG_INIT
            prev = lambda a: np.concatenate([a[:1], a[:-1]])
            r["tc"], r["tc_p1"] = prev(d["tcomov"]), d["tcomov"]
            r["m"], r["m_p1"] = prev(m), m
            r["rho"], r["rho_p1"] = prev(rho), rho
            r["u_p"], r["u_p_p1"] = prev(up), up
            gprev = prev(gsh)
            r["dr"] = prev(th) * gprev
            r["dr_p1"] = th * (gprev if is_rs else gsh)
            if first < n:
                r["dr"][first] = th[first]
            for k in ("B", "gamma_min", "gamma_max", "gamma_c", "accel_frac"):
                r[k] = lim[k]
            r["n_prime"] = ss["n_prime"]
            recs.append(r)
            params.append(shock_params(sh))
    offsets = np.zeros(len(recs) + 1, dtype=np.int64)
    offsets[1:] = np.cumsum([len(r) for r in recs])
    return np.concatenate(recs), offsets, np.array(params, dtype=abi.SHOCK_PARAMS_DTYPE)


SIGMA_T = 6.6524e-25
M_E = 9.1094e-28


def substeps(recs, offsets, params, gam):
    """Chang-Cooper substeps of every record as the step counts them
    (microphysics.h:412-435): -1 for a blastwave's first valid record (the
    initialisation), 0 for skipped records and for the analytic gamma_min <= 2
    law (:446-448), else the substep count of the record's time step."""
    n = np.zeros(len(recs), dtype=np.int64)
    dlog = (gam[1] - gam[0]) / gam[0]
    for b in range(len(params)):
        r = recs[offsets[b]:offsets[b + 1]]
        v = np.flatnonzero(r["mode"] != 0)
        if not len(v):
            continue
        out = n[offsets[b]:offsets[b + 1]]
        out[v[0]] = -1
        x = r[v[1:]]
        dt = x["tc_p1"] - x["tc"]
        with np.errstate(divide="ignore", invalid="ignore"):
            dlnv = 1.0 / dt * (1.0 - (x["m"] / x["rho"]) / (x["m_p1"] / x["rho_p1"]))
            if not params[b]["adi_on"]:
                dlnv = np.zeros_like(dt)
            dts = SIGMA_T * x["gamma_max"] * x["B"] ** 2 / (6.0 * np.pi * M_E * C_LIGHT)
            dta = (x["gamma_max"] ** 2 - 1.0) / (3.0 * x["gamma_max"] ** 2) * dlnv
            d = dlog / (dts + dta)
            ms = int(params[b]["max_substeps"])
            k = np.where(d >= dt, 1, np.where(d < dt / ms, ms, np.floor(dt / np.where(d > 0, d, 1.0))))
        k = np.where(x["gamma_min"] <= 2.0, 0, k)
        if params[b]["ele_method"] == abi.PBAG_ELE_MIX:
            k[:] = 0
        out[v[1:]] = k.astype(np.int64)
    return n


def split_chain(recs, offsets, params, gam):
    """The blastwaves' Chang-Cooper chains and the rest: (chain, rest) where
    chain = (recs, offsets, params) of every blastwave with Chang-Cooper
    records, cut after its last one, and rest = (recs, offsets, params) of
    every other valid record as a one-step blastwave. A timing aid: the
    chain is the part of a batch whose steps depend on one another through
    N(gamma); the rest still depends on its previous step through the photon
    field when SSC is on, so the one-step form computes other numbers."""
    ns = substeps(recs, offsets, params, gam)
    cr, cl, cp, rest = [], [], [], []
    for b in range(len(params)):
        cc = np.flatnonzero(ns[offsets[b]:offsets[b + 1]] > 0)
        end = int(cc[-1]) + 1 if len(cc) else 0
        if end:
            cr.append(recs[offsets[b]:offsets[b] + end])
            cl.append(end)
            cp.append(params[b])
        rest.extend(range(offsets[b] + end, offsets[b + 1]))
    co = np.zeros(len(cl) + 1, dtype=np.int64)
    co[1:] = np.cumsum(cl)
    chain = (np.concatenate(cr) if cr else recs[:0], co, np.array(cp, dtype=abi.SHOCK_PARAMS_DTYPE))
    rest = np.array(rest, dtype=np.int64)
    rest = rest[recs["mode"][rest] != 0]
    bw = np.searchsorted(offsets, rest, side="right") - 1
    return chain, (recs[rest].copy(), np.arange(len(rest) + 1, dtype=np.int64), params[bw])


# the saved dynamics (BW::VARNAMES) each pbag_eats_q quantity is read from
DRIVER_EATS_Q = {"tburst": "tburst", "R": "R", "theta": "theta", "Gamma": "Gamma", "beta": "beta",
                 "GammaFsh": "GammaFsh", "thickness": "thickness", "M2": "M2", "rho2": "rho2", "Rsh": "Rsh",
                 "acc_frac": "accel_frac", "ctheta": "ctheta", "GammaRsh": "GammaRsh",
                 "thickness_rs": "thichness_rs", "M3": "M3", "rho3": "rho3", "Rrsh": "Rsh_rs",
                 "acc_frac_rs": "accel_frac_rs"}


def driver_eats_inputs(dyn, theta_wing, rs):
    """The layer table and the EATS dynamics of a jet from the dynamics its
    ODE driver saved, as the reference's adaptive light curve reads them
    (Ejecta::computeEjectaLightCurve, ejecta_base.h:1160-1190 over
    EATS::evalFluxDensA, eats.h:823-850): layer l spans theta_pw[l] ..
    theta_pw[l+1], theta_pw[i] = 2 asin(i / nlayers sin(theta_wing / 2)) -
    the 1D initial data's loader sets up the adaptive grid and then the
    piece-wise one over it (EjectaID2::_init_pw_grid, ejecta_id.h:161-181,
    called after _init_a_grid at :293-296), so the piece-wise edges are the
    ones the light curve reads; its histories end at the first R == 0
    (checkEvolutionEnd, blastwave.h:243-253). Blastwave numbering as
    driver_records: 2 l and 2 l + 1 with the reverse shock, l without.
    Returns (layers, dyn [nlayers][PBAG_EQ_N][nr])."""
    nl = len(dyn)
    nr = len(dyn[0]["tburst"])
    layers = np.zeros(nl, dtype=abi.EATS_LAYER_DTYPE)
    out = np.zeros((nl, abi.PBAG_EQ_N, nr))
    edge = [2.0 * np.arcsin(i / nl * np.sin(theta_wing / 2.0)) for i in range(nl + 1)]
    per = 2 if rs else 1
    for il, d in enumerate(dyn):
        for iq, q in enumerate(abi.EATS_Q):
            src = DRIVER_EATS_Q[q]
            if src in d:
                out[il, iq] = d[src]
        zero = np.flatnonzero(d["R"] == 0.0)
        i_end = int(zero[0]) if len(zero) else nr
        has_rs = rs and "U_p3" in d  # no reverse shock below min_Gamma0_for_rs
        layers[il] = (i_end, per * il, per * il + 1 if has_rs else -1, 0, edge[il], edge[il + 1], 1.0)
    return layers, out


# the parfile's microphysics methods of a recorded run (method_gamma_min
# useNumeric, method_gamma_c useTcomov, method_gamma_max useB, method_B
# useU_b, method_nonrel_dist use_Sironi) and max_substeps
DRIVER_METHODS = dict(method_gamma_min=1, method_gamma_c=1, method_gamma_max=0, method_B=0, method_nonrel=3,
                      max_substeps=2000)


class DriverRun:
    """A run of the reference's own program recorded to an .npz (the dynamics
    its blastwave driver saved, saveEjectaBWsDynamics; the comoving spectra
    its step wrote, computeSaveEjectaSpectrum; its adaptive-EATS light curve,
    computeSaveEjectaLightCurve; the run's options): grid, per-layer
    dynamics, shock options, the reference's spectra
    (spec[(layer, "fs"|"rs", "j"|"a")], every `every`-th time index) and
    light curve (lc [nlayers][ntimes])."""

    def __init__(self, path):
        z = np.load(path)
        g = z["grid"]
        self.grid = abi.GridDesc(int(g[0]), int(g[1]), g[2], g[3], g[4], g[5])
        self.nlayers = int(z["layers"])
        # per layer the quantities its blastwave saved (no reverse-shock ones
        # where the driver ran none)
        self.dyn = [{k.split("_", 1)[1]: z[k] for k in z.files if k.startswith(f"dyn{il}_")}
                    for il in range(self.nlayers)]
        self.rs = bool(z["opt_rs"])
        ssc, ssa = bool(z["opt_ssc"]), bool(z["opt_ssa"])
        fs = Shock(eps_e=float(z["par_eps_e_fs"]), eps_b=float(z["par_eps_b_fs"]), p=float(z["par_p_fs"]),
                   ssc=ssc, ssa=ssa, **DRIVER_METHODS)
        rs = Shock(eps_e=float(z["par_eps_e_rs"]), eps_b=float(z["par_eps_b_rs"]), p=float(z["par_p_rs"]),
                   ssc=ssc, ssa=ssa, **DRIVER_METHODS) if self.rs else None
        self.shocks = (fs, rs)
        self.every = int(z["spec_every"])
        self.spec = {}
        for k in z.files:
            if k.startswith("spec") and k[4].isdigit():
                il, rest = k[4:].split("_", 1)           # "<il>_total_<q>_<shock>"
                _, q, shock = rest.split("_")
                self.spec[(int(il), shock, q)] = z[k]
        self.theta_wing = float(z["id_theta_wing"])
        self.theta_obs, self.z, self.d_l = float(z["par_theta_obs"]), float(z["par_z"]), float(z["par_d_l"])
        self.lc_times, self.lc_freqs = z["lc_times"], z["lc_freqs"]
        self.lc = np.array([z[f"lc{il}"] for il in range(self.nlayers)])

    def blastwave(self, il, shock):
        """Index of (layer, "fs"|"rs") among driver_records' blastwaves."""
        return (2 * il + (shock == "rs")) if self.rs else il

    def records(self, tables, layers=None):
        """driver_records over the first `layers` layers (all by default);
        tables: what provides grids and shock_limits (the library, or the
        oracle where the library must not be loaded)."""
        gam, _ = tables.grids(self.grid)
        dyn = self.dyn if layers is None else self.dyn[:layers]
        return driver_records(tables, dyn, self.shocks, gam)

    def eats_opts(self):
        """The parfile's EATS options: CADRE, counter jet, rtol 1e-6 and
        nmax 1000 in theta and phi, method_vel sameAsBW, method_ne useNe,
        method_tau smooth."""
        o = abi.EatsOpts()
        o.theta_obs, o.z, o.d_l = self.theta_obs, self.z, self.d_l
        o.rtol_theta = o.rtol_phi = 1e-6
        o.nmax_theta = o.nmax_phi = 1000
        o.method_quad = abi.PBAG_QUAD_CADRE
        o.counter_jet = 1
        o.flux.shock_vel = abi.PBAG_VEL_SAME_AS_BW
        o.flux.method_ne, o.flux.method_tau = abi.PBAG_NE_USE_NE, abi.PBAG_TAU_SMOOTH
        return o

    def eats(self):
        """(layers, dyn, queries): every layer at every light-curve time."""
        layers, dyn = driver_eats_inputs(self.dyn, self.theta_wing, self.rs)
        nt = len(self.lc_times)
        q = np.zeros(self.nlayers * nt, dtype=abi.EATS_QUERY_DTYPE)
        for il in range(self.nlayers):
            for k in range(nt):
                q[il * nt + k] = (il, 0, self.lc_times[k], self.lc_freqs[k])
        return layers, dyn, q


def eats_inputs(cfg, recs, offsets, nsteps=None):
    """The dynamics each layer's EATS reads (pbag_eats_q order), from the same
    thin-shell model make_batch records, and the layer table: (layers
    [nlayers] EATS_LAYER_DTYPE, dyn [nlayers][PBAG_EQ_N][nr]). recs / offsets:
    make_batch's records of the jet (their accel_frac; blastwave 2 l is layer
    l's forward shock and 2 l + 1 its reverse shock when cfg.rs is set). The
    jet does not spread: the edge theta is the layer's upper cone angle."""
    tb = np.logspace(np.log10(cfg.tb1), np.log10(cfg.tb2), cfg.ntb)
    if nsteps is not None:
        tb = tb[:nsteps]
    nr = len(tb)
    lo, hi, E, G0 = layer_table(cfg)
    omega = 2 * np.pi * (np.cos(lo) - np.cos(hi)) * 2
    dynl = layer_dynamics_many(E, G0, cfg.n_ism, tb, omega)
    per = 2 if cfg.rs is not None else 1
    layers = np.zeros(cfg.nlayers, dtype=abi.EATS_LAYER_DTYPE)
    dyn = np.zeros((cfg.nlayers, abi.PBAG_EQ_N, nr))
    q = {k: i for i, k in enumerate(abi.EATS_Q)}
    for il in range(cfg.nlayers):
        d = dynl[il]
        fs = fs_state(d)
        b = per * il
        acc = recs["accel_frac"][offsets[b]:offsets[b + 1]]
        row = dyn[il]
        row[q["tburst"]], row[q["R"]], row[q["Rsh"]] = tb, d["R"], d["R"]
        row[q["theta"]], row[q["ctheta"]] = hi[il], 0.5 * (lo[il] + hi[il])
        row[q["Gamma"]], row[q["beta"]], row[q["GammaFsh"]] = d["Gamma"], d["beta"], fs["GammaSh"]
        row[q["thickness"]], row[q["M2"]], row[q["rho2"]] = fs["thick"], fs["m2"], fs["rho2"]
        row[q["acc_frac"]] = np.where(acc > 0, acc, 1.0)
        layers[il] = (nr, b, b + 1 if per == 2 else -1, 0, lo[il], hi[il], 1.0)
        if per == 2:
            rs = rs_state(d)
            acr = recs["accel_frac"][offsets[b + 1]:offsets[b + 2]]
            # reverse-shock radiation only where its shell exists (thickness > 0 at both ends of a segment)
            row[q["GammaRsh"]], row[q["Rrsh"]] = rs["GammaSh"], d["R"]
            row[q["thickness_rs"]] = np.where(rs["valid"], rs["thick"], 0.0)
            row[q["M3"]], row[q["rho3"]] = rs["m2"], rs["rho2"]
            row[q["acc_frac_rs"]] = np.where(acr > 0, acr, 1.0)
    return layers, dyn


def driver_arrays(lib, cfg, nsteps=None):
    """Per blastwave (ordered as make_batch orders them) the quantities the
    reference's blastwave driver passes to ElectronAndRadiation at every
    burster time (blastwave_radiation.h:976-1182): a list of (is_rs, dict of
    arrays) with valid, U_p, Gamma, GammaSh, t_e, t_b, tcomov, n_prime,
    n_protons, M2, rho2, R, thickness (passed at the first valid step) and the
    comoving thickness (passed to the evolution). `valid` marks the steps
    make_batch records (the driver skips the others)."""
    tb = np.logspace(np.log10(cfg.tb1), np.log10(cfg.tb2), cfg.ntb)
    if nsteps is not None:
        tb = tb[:nsteps]
    gam, _ = lib.grids(cfg.grid())
    lo, hi, E, G0 = layer_table(cfg)
    omega = 2 * np.pi * (np.cos(lo) - np.cos(hi)) * 2
    dyn = layer_dynamics_many(E, G0, cfg.n_ism, tb, omega)
    out = []
    for il in range(cfg.nlayers):
        d = dyn[il]
        for is_rs, st, sh in ((False, fs_state(d), cfg.fs), (True, rs_state(d) if cfg.rs is not None else None, cfg.rs)):
            if st is None:
                continue
            ss = np.zeros(len(tb), dtype=abi.SHOCK_STATE_DTYPE)
            ss["e_prime"], ss["Gamma"], ss["GammaSh"] = st["u_p"], st["Gamma"], st["GammaSh"]
            ss["t_e"], ss["t_b"], ss["tcomov"] = d["t_obs"], tb, d["tcomov"]
            ss["n_prime"], ss["n_protons"] = st["rho2"] / M_P, st["m2"] / M_P
            lim = lib.shock_limits(limits_opts(sh), gam, ss)
            valid = st["valid"] & (lim["valid"] == 1) & (st["u_p"] > 0) & (st["rho2"] > 0)
            out.append((is_rs, dict(valid=valid.astype(np.float64), U_p=st["u_p"], Gamma=st["Gamma"],
                                    GammaSh=st["GammaSh"], t_e=d["t_obs"], t_b=tb, tcomov=d["tcomov"],
                                    n_prime=st["rho2"] / M_P, n_protons=st["m2"] / M_P, M2=st["m2"],
                                    rho2=st["rho2"], R=d["R"], thickness=st["thick"], dr=st["dr"])))
    return out


def _sweep_set(cfg):
    from . import _lib
    return make_batch(_lib, cfg)


def sweep_batch(lib, nsets, seed=3, ngam=201, nfreq=128, min_steps=200, max_steps=2000, ssc=True,
                max_layers=41, workers=1, first=0):
    """Seeded parameter sweep: nsets jets, each a top-hat or Gaussian with
    1..max_layers layers, log10 E_iso ~ U[50,54], log10 Gamma0 ~ U[1,3],
    log10 n ~ U[-4,0], log10 eps_e ~ U[-3,-0.5], log10 eps_b ~ U[-5,-1],
    p ~ U[2.05,2.8]; every blastwave keeps its first U{min_steps..max_steps}
    steps (uneven histories). first: index of the first set in the seeded
    sequence (sets first .. first+nsets-1 of the same sweep, so that ranks
    can take disjoint shards of it). workers > 1 builds the jets in a process
    pool (spawned, so it is safe next to a CUDA context)."""
    rng = np.random.default_rng(seed)
    cfgs, counts = [], []
    for i in range(first + nsets):
        struct = "tophat" if rng.random() < 0.5 else "gaussian"
        nl = int(rng.integers(1, max_layers + 1))
        sh = dict(eps_e=10 ** rng.uniform(-3, -0.5), eps_b=10 ** rng.uniform(-5, -1),
                  p=rng.uniform(2.05, 2.8), ssc=ssc, ssa=True)
        tc = rng.uniform(0.05, 0.15)
        cfg = JetConfig(struct=struct, E_iso=10 ** rng.uniform(50, 54),
                        Gamma0=10 ** rng.uniform(1, 3), theta_c=tc, theta_w=min(4 * tc, 0.6),
                        n_ism=10 ** rng.uniform(-4, 0), nlayers=nl, fs=Shock(**sh), rs=Shock(**sh),
                        ngam=ngam, gam1=1.0, gam2=1e9, nfreq=nfreq, ntb=max_steps)
        cnt = [int(rng.integers(min_steps, max_steps + 1)) for _ in range(2 * nl)]
        if i >= first:
            cfgs.append(cfg)
            counts.append(cnt)
    if workers > 1 and nsets > 1:
        import multiprocessing as mp
        with mp.get_context("spawn").Pool(min(workers, nsets)) as pool:
            batches = pool.map(_sweep_set, cfgs)
    else:
        batches = [make_batch(lib, c) for c in cfgs]
    all_recs, params, lens = [], [], []
    grid = None
    for (recs, off, prm, grid), cnt in zip(batches, counts):
        for b in range(len(off) - 1):
            r = recs[off[b]:off[b] + cnt[b]]
            all_recs.append(r)
            lens.append(len(r))
            params.append(prm[b])
    offsets = np.zeros(len(lens) + 1, dtype=np.int64)
    offsets[1:] = np.cumsum(lens)
    return np.concatenate(all_recs), offsets, np.array(params, dtype=abi.SHOCK_PARAMS_DTYPE), grid
