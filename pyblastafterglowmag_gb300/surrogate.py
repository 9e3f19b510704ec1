"""Training and deployment of the SSC surrogate (pbag_surrogate_* and the
library's own MLP kernels, pbag_mlp_*).

Data: comoving states (N(gamma) after a step, B, the photon field of the
previous radiating step) of seeded blastwaves from the batched parameter sweep,
evolved by the plain GPU step. Targets: log10 of each frequency's share of its
band's power in the exact SSC spectrum (pbag_contract, split BF16) minus the
baseline share (the log-parabola matched to the band's exact power, first and
second moments), weighted by emissivity (zero where the band carries no
power). Features, the exact projections and the baseline come from
pbag_surrogate_features. The network: PBAG_SUR_IN -> 4 x 256 (SiLU) -> nfreq,
trained in FP32 with Adam on weighted squared error by the library's kernels,
run in BF16 on the tensor cores. The
error estimate's scale is calibrated on held-out states against the exact
spectra (calibrate).
"""
import ctypes as C
import math

import numpy as np

from . import _lib, abi
from . import histories as H
from .mlp import MLP

NIN, NB, NCHK = 128, 16, 32
NPROJ = 3 * NB + NCHK
HIDDEN = (256, 256, 256, 256)
TARGET_FLOOR = -12.0
WEIGHT_FLOOR = 1e-3


def _bind():
    lib = _lib.load()
    if not getattr(lib, "_sur_bound", False):
        P = C.POINTER
        lib.pbag_surrogate_configure.argtypes = [C.c_void_p, C.c_void_p, P(C.c_float), P(C.c_float), C.c_float,
                                                 C.c_float]
        lib.pbag_surrogate_checks.argtypes = [C.c_void_p, P(C.c_int)]
        lib.pbag_surrogate_features.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                                                C.c_void_p, C.c_void_p, C.c_void_p, P(abi.Status)]
        lib.pbag_surrogate_contract.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                                                C.c_void_p, C.c_void_p, P(C.c_int), P(abi.Status)]
        lib._sur_bound = True
    return lib


def configure(ctx, net=None, mean=None, std=None, tol=0.01, est_scale=1.0):
    lib = _bind()
    m = None if mean is None else np.ascontiguousarray(mean, dtype=np.float32)
    s = None if std is None else np.ascontiguousarray(std, dtype=np.float32)
    fp = lambda a: None if a is None else a.ctypes.data_as(C.POINTER(C.c_float))
    _lib._check(lib.pbag_surrogate_configure(ctx.handle, net.handle if net is not None else None,
                                             fp(m), fp(s), float(est_scale), float(tol)),
                "pbag_surrogate_configure")


def checks(ctx):
    """Frequency index of each check projection (columns 3 NB .. NPROJ of the projections)."""
    idx = (C.c_int * NCHK)()
    _lib._check(_bind().pbag_surrogate_checks(ctx.handle, idx), "pbag_surrogate_checks")
    return np.array(idx[:], dtype=np.int64)


def features(ctx, n, d_f, d_B, d_nph, d_x, d_proj, d_base=0):
    st = abi.Status()
    _lib._check(_bind().pbag_surrogate_features(ctx.handle, int(n), C.c_void_p(d_f), C.c_void_p(d_B),
                                                C.c_void_p(d_nph), C.c_void_p(d_x or None),
                                                C.c_void_p(d_proj or None), C.c_void_p(d_base or None),
                                                C.byref(st)),
                "pbag_surrogate_features", st)


def contract(ctx, n, d_f, d_B, d_nph, d_jssc, d_err=0):
    st = abi.Status()
    nfb = C.c_int()
    _lib._check(_bind().pbag_surrogate_contract(ctx.handle, int(n), C.c_void_p(d_f), C.c_void_p(d_B),
                                                C.c_void_p(d_nph), C.c_void_p(d_jssc), C.c_void_p(d_err or None),
                                                C.byref(nfb), C.byref(st)), "pbag_surrogate_contract", st)
    return int(nfb.value)


def sweep_states(ctx, grid, nsets, seed=5, workers=1, device=0, max_states=None):
    """States (f [n][G], B [n], photon field [n][F]) of every radiating step
    after the first of each blastwave of a seeded sweep, evolved by the plain
    GPU step (torch tensors on the device)."""
    import torch
    recs, off, prm, g = H.sweep_batch(_lib, nsets, seed=seed, ngam=grid.ngam, nfreq=grid.nfreq, workers=workers)
    dev = torch.device("cuda", device)
    nrec, G, F = len(recs), grid.ngam, grid.nfreq
    d_recs = torch.from_numpy(recs.view(np.uint8).copy()).to(dev)
    d_prm = torch.from_numpy(prm.view(np.uint8).copy()).to(dev)
    d_ef = torch.zeros((nrec, G), dtype=torch.float64, device=dev)
    d_nf = torch.zeros((nrec, F), dtype=torch.float64, device=dev)
    try:
        ctx.run_device(d_prm.data_ptr(), len(prm), off, d_recs.data_ptr(),
                       {"ele_f_all": d_ef.data_ptr(), "f_all": d_nf.data_ptr()})
    except _lib.PbagError:
        pass  # a failing blastwave keeps its rows up to the failure; its later rows stay zero
    # pair every radiating row with the photon field of the blastwave's previous radiating row
    ef = d_ef.abs().sum(dim=1) > 0
    rad = (d_nf.abs().sum(dim=1) > 0) & ef
    rad_h = rad.cpu().numpy()
    idx_now, idx_prev = [], []
    for b in range(len(prm)):
        rows = np.nonzero(rad_h[off[b]:off[b + 1]])[0] + off[b]
        idx_now.append(rows[1:])
        idx_prev.append(rows[:-1])
    now = np.concatenate(idx_now)
    prev = np.concatenate(idx_prev)
    if max_states is not None and len(now) > max_states:
        pick = np.random.default_rng(seed).choice(len(now), max_states, replace=False)
        now, prev = now[pick], prev[pick]
    t_now = torch.from_numpy(now).to(dev)
    t_prev = torch.from_numpy(prev).to(dev)
    f = d_ef[t_now].contiguous()
    nph = d_nf[t_prev].contiguous()
    B = torch.from_numpy(np.ascontiguousarray(recs["B"][now])).to(dev)
    return f, B, nph


def exact_ssc(ctx, f, B, nph):
    import torch
    n, F = f.shape[0], nph.shape[1]
    j = torch.zeros((n, F), dtype=torch.float64, device=f.device)
    ctx.contract_device(n, f.data_ptr(), B.data_ptr(), nph.data_ptr(), abi.PBAG_SYN_CSYN,
                        abi.PBAG_PREC_SPLIT_BF16, 0, j.data_ptr())
    return j


def make_targets(jssc, proj, freq, base):
    """The network's targets: log10 of each frequency's share of its band's
    exact power minus the baseline share (the log-parabola matched to the
    band's exact moments), and the loss weights (zero where the band carries
    no power or the share is below the floor)."""
    import torch
    n, F = jssc.shape
    per = F // NB
    nu = torch.from_numpy(np.asarray(freq)).to(jssc.device)
    dnu = (nu[1:F + 1] - nu[:F])[None, :]
    P = proj[:, :NB].repeat_interleave(per, dim=1)
    share = jssc * dnu / torch.where(P > 0, P, torch.ones_like(P))
    t = torch.log10(torch.clamp(share, min=10.0 ** TARGET_FLOOR)).clamp(min=TARGET_FLOOR, max=1.0)
    t = (t - base.to(t.dtype)).clamp(min=-12.0, max=12.0)
    # frequencies below the floor carry no power that matters; left unmasked
    # they would dominate the loss with large, meaningless corrections
    mask = ((P > 0) & (share > 10.0 ** TARGET_FLOOR)).to(torch.float32)
    # weights: the relative L2 error of a spectrum is dominated by its
    # brightest frequencies, so each frequency counts with its emissivity
    # (normalised to a mean of one per state), plus a small floor
    a = jssc.abs()
    w = (a / torch.clamp(a.sum(dim=1, keepdim=True), min=1e-300) * F).to(torch.float32)
    return t.to(torch.float32).contiguous(), ((w + WEIGHT_FLOOR) * mask).contiguous()


def band_baseline(proj, freq, base):
    """The method without the network: in each band the baseline shape (the tilt
    matched to the band's exact power and first moment) scaled to the power."""
    import torch
    F = len(freq) - 1
    per = F // NB
    nu = torch.from_numpy(np.asarray(freq)).to(proj.device)
    dnu = (nu[1:F + 1] - nu[:F])[None, :]
    share = torch.pow(10.0, base.to(torch.float64))
    return proj[:, :NB].clamp(min=0).repeat_interleave(per, dim=1) * share / dnu


def rel_l2_rows(x, y):
    """Relative L2 error of every row (NaN where the reference row is zero)."""
    import torch
    num = torch.sqrt(((x - y) ** 2).sum(dim=1))
    den = torch.sqrt((y ** 2).sum(dim=1))
    return torch.where(den > 0, num / torch.where(den > 0, den, torch.ones_like(den)),
                       torch.full_like(den, float("nan")))


def calibrate(ctx, trainer, f, B, nph, jex, quantile=0.95):
    """Scale of the error estimate: the given quantile, over held-out states,
    of the true relative L2 error divided by the unscaled estimate (the
    distance at the check frequencies). Leaves the surrogate configured with
    that scale and no fallback."""
    import torch
    configure(ctx, trainer.net, trainer.mean, trainer.std, tol=1e30, est_scale=1.0)
    n = f.shape[0]
    j = torch.zeros_like(jex)
    est = torch.zeros(n, dtype=torch.float32, device=f.device)
    contract(ctx, n, f.data_ptr(), B.data_ptr(), nph.data_ptr(), j.data_ptr(), est.data_ptr())
    err = rel_l2_rows(j, jex)
    ok = torch.isfinite(err)
    ratio = err[ok] / torch.clamp(est[ok].double(), min=1e-12)
    scale = float(torch.quantile(ratio.float(), quantile)) if ratio.numel() else 1.0
    scale = max(scale, 1e-3)
    configure(ctx, trainer.net, trainer.mean, trainer.std, tol=1e30, est_scale=scale)
    return scale


def rel_l2(x, y):
    import torch
    num = torch.sqrt(((x - y) ** 2).sum(dim=1))
    den = torch.sqrt((y ** 2).sum(dim=1))
    ok = den > 0
    return (num[ok] / den[ok])


class Trainer:
    """Trains the network of the surrogate on device tensors."""

    def __init__(self, nfreq, device=0, seed=0):
        self.dims = [NIN, *HIDDEN, nfreq]
        self.net = MLP(self.dims, device)
        self.net.init_params(seed=seed)
        self.mean = np.zeros(NIN, dtype=np.float32)
        self.std = np.ones(NIN, dtype=np.float32)

    def standardise(self, X):
        """Feature means and deviations from the training set; X standardised in place."""
        import torch
        m = X.mean(dim=0)
        s = X.std(dim=0)
        s = torch.where(s > 1e-6, s, torch.ones_like(s))
        self.mean = m.cpu().numpy().astype(np.float32)
        self.std = s.cpu().numpy().astype(np.float32)
        X.sub_(m[None, :]).div_(s[None, :])
        return X

    def fit(self, X, T, M, epochs=20, batch=4096, lr=1e-3, seed=0, log=None):
        import torch
        n = X.shape[0]
        steps = max(1, epochs * (n // batch))
        g = torch.Generator(device=X.device)
        g.manual_seed(seed)
        loss = None
        step = 0
        for ep in range(epochs):
            perm = torch.randperm(n, device=X.device, generator=g)
            for s0 in range(0, n - batch + 1, batch):
                idx = perm[s0:s0 + batch]
                xb, tb, mb = X[idx].contiguous(), T[idx].contiguous(), M[idx].contiguous()
                rate = lr * 0.5 * (1 + math.cos(math.pi * step / steps))
                loss = self.net.train_step(batch, xb.data_ptr(), tb.data_ptr(), mb.data_ptr(), lr=rate)
                step += 1
            if log:
                log(ep, loss)
        return loss

    def state(self):
        return {"dims": np.array(self.dims), "params": self.net.params(), "mean": self.mean, "std": self.std}
