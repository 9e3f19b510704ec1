"""Per-step shock scalars on the GPU (pbag_shock_limits_device) against the
values the reference produced (tests/golden/shock_limits.npz: every
gamma_min, gamma_c, gamma_max, B and non-relativistic method) and against the
host prep called state after state (pbag_shock_limits) on the full Gaussian
jet's histories and on histories with refused states (beta_shock below
beta_min) interleaved, where the members carry over. Tolerance: relative
1e-12 (device pow / log against the host's); the useNumeric bisection may
move by one of its 0.1 % steps on a rounding tie and is checked at that
granularity."""
import os

import numpy as np
import pytest

from pyblastafterglowmag_gb300 import abi, histories as H

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLD = os.path.join(ROOT, "tests", "golden")
COLS = ["B", "gamma_min", "gamma_max", "gamma_c", "accel_frac", "Theta", "z_cool"]


def _opts(gm, gc, gx, bm, nr, p):
    o = abi.LimitsOpts()
    o.p, o.eps_e, o.eps_b, o.eps_t = p, 0.1, 1e-3, 0.5
    o.beta_min, o.mu, o.mu_e = 1e-5, 0.62, 1.18
    o.method_B, o.method_gamma_min, o.method_gamma_c = int(bm), int(gm), int(gc)
    o.method_gamma_max, o.method_nonrel, o.ele_analytic = int(gx), int(nr), 0
    return o


def _run_device(lib, ctx, opts_list, states_list, state0):
    import torch
    nbw = len(opts_list)
    off = np.zeros(nbw + 1, dtype=np.int64)
    off[1:] = np.cumsum([len(s) for s in states_list])
    ob = b"".join(bytes(o) for o in opts_list)
    d_opts = torch.frombuffer(bytearray(ob), dtype=torch.uint8).cuda()
    ins = np.concatenate(states_list).astype(abi.SHOCK_STATE_DTYPE)
    d_in = torch.from_numpy(ins.view(np.uint8).copy()).cuda()
    d_state = torch.from_numpy(np.ascontiguousarray(state0, dtype=np.float64)).cuda()
    d_out = torch.zeros(int(off[-1]) * abi.LIMITS_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    lib.shock_limits_device(ctx, off, d_opts.data_ptr(), d_in.data_ptr(), d_state.data_ptr(), d_out.data_ptr())
    out = d_out.cpu().numpy().view(abi.LIMITS_DTYPE)
    return [out[off[b]:off[b + 1]] for b in range(nbw)], d_state.cpu().numpy()


def _stack(x):
    return np.stack([x[c] for c in COLS] + [x["valid"].astype(float)], axis=1)


def _close(got, ref, numeric):
    if not numeric:
        np.testing.assert_allclose(got, ref, rtol=1e-12, atol=0)
        return
    same = np.isclose(got, ref, rtol=1e-12, atol=0).all(axis=1)
    assert same.mean() >= 0.9, same.mean()
    np.testing.assert_allclose(got, ref, rtol=2.5e-3, atol=0)


def test_device_limits_match_reference_fixture(lib, cuda_device):
    d = np.load(os.path.join(GOLD, "shock_limits.npz"))
    a = d["grid"]
    grid = abi.GridDesc(int(a[0]), int(a[1]), *map(float, a[2:]))
    ctx = lib.Context(grid, cuda_device, ssc=False)
    opts = [_opts(*o) for o in d["opts"]]
    state0 = np.array([[-1.0, 1e7, 1e5 if int(o[1]) == 2 else -1.0, 1.0, -1.0, -1.0, -1.0] for o in d["opts"]])
    got, _ = _run_device(lib, ctx, opts, [d["states"]] * len(opts), state0)
    for o, g, ref in zip(d["opts"], got, d["out"]):
        _close(_stack(g), ref, numeric=int(o[0]) == 1)
    ctx.close()


def test_device_limits_match_host_with_refused_states(lib, cuda_device):
    """States with beta_shock below beta_min leave every member as it was, and
    accel_frac keeps the value of the last state that assigned it: the device's
    carries reproduce the host's call-after-call members."""
    d = np.load(os.path.join(GOLD, "shock_limits.npz"))
    a = d["grid"]
    grid = abi.GridDesc(int(a[0]), int(a[1]), *map(float, a[2:]))
    gam, _ = lib.grids(grid)
    rng = np.random.default_rng(21)
    st = np.concatenate([d["states"]] * 3).copy()
    refuse = rng.random(len(st)) < 0.3
    refuse[:5] = True  # refused states before the first accepted one
    st["GammaSh"][refuse] = 1.0 + 1e-12
    ctx = lib.Context(grid, cuda_device, ssc=False)
    opts = [_opts(*o) for o in d["opts"]]
    state0 = np.array([[-1.0, 1e7, 1e5 if int(o[1]) == 2 else -1.0, 1.0, -1.0, -1.0, -1.0] for o in d["opts"]])
    got, st_dev = _run_device(lib, ctx, opts, [st] * len(opts), state0)
    for b, (o, g) in enumerate(zip(d["opts"], got)):
        s0 = state0[b].copy()
        ref = lib.shock_limits(opts[b], gam, st, state=s0)
        _close(_stack(g), _stack(ref), numeric=int(o[0]) == 1)
        assert (g["valid"] == ref["valid"]).all() and not g["valid"][refuse].any()
        np.testing.assert_allclose(st_dev[b], s0, rtol=2.5e-3 if int(o[0]) == 1 else 1e-12)
    ctx.close()


def test_device_limits_full_jet(lib, cuda_device):
    """All 42 blastwaves x 1000 burster times of the Gaussian jet: the device
    prep equals the host prep the batch generator uses."""
    cfg = H.config_gaussian_ssc()
    grid = cfg.grid()
    gam, _ = lib.grids(grid)
    tb = np.logspace(np.log10(cfg.tb1), np.log10(cfg.tb2), cfg.ntb)
    lo, hi, E, G0 = H.layer_table(cfg)
    dyn = H.layer_dynamics_many(E, G0, cfg.n_ism, tb, 2 * np.pi * (np.cos(lo) - np.cos(hi)) * 2)
    states, opts, refs = [], [], []
    for il in range(cfg.nlayers):
        dd = dyn[il]
        for stt, sh in ((H.fs_state(dd), cfg.fs), (H.rs_state(dd), cfg.rs)):
            ss = np.zeros(len(tb), dtype=abi.SHOCK_STATE_DTYPE)
            ss["e_prime"], ss["Gamma"], ss["GammaSh"] = stt["u_p"], stt["Gamma"], stt["GammaSh"]
            ss["t_e"], ss["t_b"], ss["tcomov"] = dd["t_obs"], tb, dd["tcomov"]
            ss["n_prime"], ss["n_protons"] = stt["rho2"] / H.M_P, stt["m2"] / H.M_P
            states.append(ss)
            opts.append(H.limits_opts(sh))
            refs.append(lib.shock_limits(opts[-1], gam, ss))
    ctx = lib.Context(grid, cuda_device, ssc=False)
    state0 = np.tile(np.array([-1.0, 1e7, -1.0, 1.0, -1.0, -1.0, -1.0]), (len(opts), 1))
    got, _ = _run_device(lib, ctx, opts, states, state0)
    for g, r in zip(got, refs):
        np.testing.assert_allclose(_stack(g), _stack(r), rtol=1e-12, atol=0)
    ctx.close()
