"""Learned macro step of the particle-field path (no reference counterpart).

A macro step advances phi over K substeps of dt:

    phi(t + K dt) = L_K[phi(t), mu(t)] + norm[6] * C(phi(t), rho(t), chi)

L_K is the context's own step in macro mode (phafd_set_linear_substeps): K
Model-B substeps linearised about the mean concentration with the nonlinear
part of mu (Flory-Huggins remainder and bead deposit) frozen at t, the noise
of K substeps, and K bead substeps of dt against the field of time t.  C is the spectral neural
operator of include/phafd_fno.h (zero mean, so the macro step conserves
mass exactly).  The network learns R = phi_plain(t + K dt) - L_K[phi(t)],
the part of K plain substeps that the linearised step misses, on states of
trajectories that the plain FP32 integrator generates.

The plain step is the judge and the fallback: every `judge_every` substeps
the state is copied into two noise-free contexts, one advanced by K plain
substeps and one by the macro step; when the relative S(k) error or the mass
error of the macro step exceeds its bound the run drops the surrogate and
continues with plain steps.

Device buffers are torch CUDA tensors (plumbing only); every computation
runs in libphafd_gpu.so.
"""
import math
import multiprocessing as mp
import time

import numpy as np

from . import workloads as W
from .fno import FNO, init_params
from .gpu import PhafdGPU

K_SUB = 20


class DevView:
    """A device array of the context as a torch tensor (no copy)."""

    def __init__(self, ptr, shape, typestr="<f4"):
        self.__cuda_array_interface__ = {"shape": tuple(shape), "typestr": typestr, "data": (int(ptr), False),
                                         "version": 2}


def field(sim, name="phi"):
    import torch
    return torch.as_tensor(DevView(sim.grid_device(name), sim.shape), device="cuda")


def fh_f2(chi, phi0, temp=1.0, volFH=1.0):
    """dmu/dphi of the Flory-Huggins chemical potential at phi0
    (fixgrid_floryhuggins.cpp:81): T/v (1/(phi (1-phi)) - 2 chi)."""
    return temp / volFH * (1.0 / (phi0 * (1.0 - phi0)) - 2.0 * chi)


def traj_cfg(n, nbeads, chi, phi0, seed, chain_len=200, noise=True):
    """A trajectory of the training/evaluation family (128^3 or 256^3 box of
    side n, chains of `chain_len` beads)."""
    nch = max(1, int(round(nbeads / chain_len)))
    return dict(W._COMMON, n=n, L=float(n), origin=-n / 2.0, phi0=float(phi0), chi=float(chi),
                grid_seed=int(seed), nchains=nch, chain_len=chain_len, chain_seed=int(seed) + 7,
                field_noise="philox" if noise else "off", bead_temp=1.0 if noise else 0.0, steps=0)


def _chains(cfg):
    return W.random_walk_chains(cfg["nchains"], cfg["chain_len"], cfg["origin"], cfg["L"], cfg["chain_seed"],
                                cfg["bond"])


def make_chains(cfgs, workers=8):
    """Chain conformations for many configurations, in spawned processes (a
    pool forked after CUDA initialisation would hang)."""
    if workers <= 1 or len(cfgs) <= 1:
        return [_chains(c) for c in cfgs]
    with mp.get_context("spawn").Pool(workers) as pool:
        return pool.map(_chains, cfgs)


def sim(cfg, chains, noise=True, device=0):
    c = dict(cfg)
    if not noise:
        c["field_noise"] = "off"
        c["bead_temp"] = 0.0
    s = PhafdGPU(precision=32, device=device, schedule="resident")
    W.apply(s, c, chains=chains)
    s.setup()
    return s


def mean_phi(s):
    return float(field(s).double().mean().item())


def rel_sk_error(sa, sb, skip=1):
    """max over shells of |S_a - S_b| / S_b (shells with modes)."""
    m = sb[skip:] > 0
    return float(np.max(np.abs(sa[skip:][m] - sb[skip:][m]) / sb[skip:][m]))


# --------------------------------------------------------------------- data
def generate(specs, samples=2, burn=200, gap=100, K=K_SUB, workers=8, log=None):
    """Training pairs from trajectories of the plain FP32 integrator.

    specs: list of (n, nbeads, chi, phi0, seed).  Per trajectory: `burn`
    noisy plain steps, then `samples` states `gap` steps apart; for each
    state the target R = phi after K noise-free plain substeps minus phi
    after the noise-free macro step without the network.
    Returns device tensors phi, rho, target [S, n, n, n], chi (numpy)."""
    import torch
    cfgs = [traj_cfg(*sp) for sp in specs]
    chains = make_chains(cfgs, workers)
    phis, rhos, tgts, chis = [], [], [], []
    t0 = time.time()
    for i, (cfg, ch) in enumerate(zip(cfgs, chains)):
        main = sim(cfg, ch, noise=True)
        jp = sim(cfg, ch, noise=False)
        jl = sim(cfg, ch, noise=False)
        jl.set_linear_substeps(K, fh_f2(cfg["chi"], cfg["phi0"]))
        main.run(burn)
        for s in range(samples):
            jp.copy_state_from(main)
            jl.copy_state_from(main)
            rho = torch.empty(main.shape, device="cuda")
            jl.deposit_density(rho.data_ptr())
            phi0 = field(jl).clone()
            jp.run(K)
            jl.run(1)
            tgts.append(field(jp) - field(jl))
            phis.append(phi0)
            rhos.append(rho)
            chis.append(cfg["chi"])
            if s + 1 < samples:
                main.run(gap)
        for s_ in (main, jp, jl):
            s_.close()
        if log and (i + 1) % max(1, len(cfgs) // 10) == 0:
            log("trajectory %d/%d (%.1f s)" % (i + 1, len(cfgs), time.time() - t0))
    return torch.stack(phis), torch.stack(rhos), torch.stack(tgts), np.array(chis, np.float32)


def norm_from(phi, rho, tgt, chis):
    """Normalisation constants of phafd_fno_set_norm from a dataset."""
    return np.array([float(phi.mean()), max(float(phi.std()), 1e-6), float(rho.mean()), max(float(rho.std()), 1e-6),
                     float(np.mean(chis)), max(float(np.std(chis)), 1e-3), max(float(tgt.std()), 1e-12), 0.0],
                    np.float32)


# --------------------------------------------------------------------- training
def train(net, data, epochs=4, lr=1e-3, batch=8, seed=0, log=None):
    """Adam on mean((out - R / norm[6])^2) over the dataset; returns the
    per-epoch mean loss."""
    import torch
    phi, rho, tgt, chis = data
    scale = float(net.norm[6])
    rng = np.random.default_rng(seed)
    hist = []
    n = phi.shape[0]
    for ep in range(epochs):
        order = rng.permutation(n)
        tot = 0.0
        for b in range(0, n, batch):
            idx = order[b:b + batch]
            net.zero_grad()
            for j in idx:
                t = (tgt[j] / scale).contiguous()
                tot += net.forward_backward(phi[j].data_ptr(), rho[j].data_ptr(), float(chis[j]), t.data_ptr())
            net.adam_step(lr, nbatch=len(idx))
        hist.append(tot / n)
        if log:
            log("epoch %d loss %.4e" % (ep, hist[-1]))
    torch.cuda.synchronize()
    return hist


def correction(net, phi, rho, chi):
    import torch
    out = torch.empty_like(phi)
    net.infer(phi.data_ptr(), rho.data_ptr(), float(chi), out.data_ptr())
    return out


def gain(net, data):
    """Relative error of the macro step with and without the network on a
    dataset: |R - C| / |R| and |R| / |R| = 1, summed over samples."""
    phi, rho, tgt, chis = data
    num = den = 0.0
    for j in range(phi.shape[0]):
        c = correction(net, phi[j], rho[j], chis[j])
        num += float(((tgt[j] - c).double() ** 2).sum())
        den += float((tgt[j].double() ** 2).sum())
    return math.sqrt(num / den)


# --------------------------------------------------------------------- runs
class Runner:
    """Production run with the learned macro step and its judge (net None:
    the linearised macro step alone, judged the same way)."""

    def __init__(self, cfg, chains, net, K=K_SUB, judge_every=100, sk_bound=1e-2, mass_bound=1e-6, nbins=None):
        import torch
        self.cfg, self.net, self.K = cfg, net, K
        self.f2 = fh_f2(cfg["chi"], cfg["phi0"])
        self.main = sim(cfg, chains, noise=True)
        self.jp = sim(cfg, chains, noise=False)
        self.js = sim(cfg, chains, noise=False)
        self.js.set_linear_substeps(K, self.f2)
        self.judge_every = judge_every
        self.sk_bound, self.mass_bound = sk_bound, mass_bound
        self.nbins = nbins or cfg["n"] // 2
        self.rho = torch.empty(self.main.shape, device="cuda")
        self.corr = torch.empty(self.main.shape, device="cuda")
        self.phi0 = torch.empty(self.main.shape, device="cuda")  # phi(t) for the network
        self.nstream = torch.cuda.Stream()
        self.corr_ready = False  # the judge's correction, valid for the main state it was copied from
        self.use_surrogate = True
        self.done = 0
        self.judged = []
        self.macro = False
        self.times = {"judge": 0.0, "density": 0.0, "network": 0.0, "step": 0.0, "add": 0.0, "plain": 0.0}

    def _t(self, key, fn, *a):
        t0 = time.perf_counter()
        fn(*a)
        self.times[key] += time.perf_counter() - t0

    def _macro(self, s, reuse=False):
        """One macro step of context s.  The network reads phi(t) and rho(t)
        only, so it runs on its own stream while the context takes the step
        (beads and the linearised field update); its correction is added
        after both.  reuse: the correction of the same state is in corr."""
        if self.net is None:  # the linearised macro step alone (the method without the network)
            self._t("step", s.run, 1)
            return
        if not reuse:
            self._t("density", s.deposit_density, self.rho.data_ptr())
            self._t("density", s.grid_copy_device, "phi", self.phi0.data_ptr())
            self._t("network", self.net.infer, self.phi0.data_ptr(), self.rho.data_ptr(), self.cfg["chi"],
                    self.corr.data_ptr(), self.nstream.cuda_stream)
        self._t("step", s.run_async, 1)
        self._t("step", s.synchronize)
        self._t("network", self.nstream.synchronize)
        self._t("add", s.grid_add_device, self.corr.data_ptr(), 1.0)

    def judge(self):
        self.jp.copy_state_from(self.main)
        self.js.copy_state_from(self.main)
        self.jp.run_async(self.K)  # the plain rerun overlaps the macro step of js
        self._macro(self.js)
        self.jp.synchronize()
        self.corr_ready = self.net is not None  # the main state is the one js started from
        sp, _ = self.jp.structure_factor(self.nbins)
        ss, _ = self.js.structure_factor(self.nbins)
        err = rel_sk_error(ss, sp)
        dm = abs(mean_phi(self.js) - mean_phi(self.jp))
        ok = err <= self.sk_bound and dm <= self.mass_bound
        self.judged.append((self.done, err, dm, ok))
        if not ok:
            self.use_surrogate = False
        return ok

    def run(self, nsteps):
        end = self.done + nsteps
        while self.done < end:
            if self.use_surrogate and self.done % self.judge_every == 0:
                self._t("judge", self.judge)
            if self.use_surrogate and end - self.done >= self.K:
                if not self.macro:
                    self.main.set_linear_substeps(self.K, self.f2)
                    self.macro = True
                self._macro(self.main, reuse=self.corr_ready)
                self.corr_ready = False
                self.done += self.K
            else:
                if self.macro:
                    self.main.set_linear_substeps(1)
                    self.macro = False
                k = min(self.K, end - self.done)
                self.corr_ready = False
                self._t("plain", self.main.run, k)
                self.done += k

    def close(self):
        for s in (self.main, self.jp, self.js):
            s.close()


def horizon_error(cfg, chains, net, horizon, K=K_SUB, nbins=None):
    """S(k) and mass of the surrogate path against the plain path after
    `horizon` substeps from the same state, both noise-free."""
    plain = sim(cfg, chains, noise=False)
    sur = sim(cfg, chains, noise=False)
    base = sim(cfg, chains, noise=False)
    f2 = fh_f2(cfg["chi"], cfg["phi0"])
    import torch
    rho = torch.empty(plain.shape, device="cuda")
    corr = torch.empty(plain.shape, device="cuda")
    plain.run(horizon)
    for s, use_net in ((sur, True), (base, False)):
        s.set_linear_substeps(K, f2)
        for _ in range(horizon // K):
            s.deposit_density(rho.data_ptr())
            if use_net:
                net.infer(s.grid_device("phi"), rho.data_ptr(), cfg["chi"], corr.data_ptr())
            s.run(1)
            if use_net:
                s.grid_add_device(corr.data_ptr(), 1.0)
    nb = nbins or cfg["n"] // 2
    sp, _ = plain.structure_factor(nb)
    ss, _ = sur.structure_factor(nb)
    sb, _ = base.structure_factor(nb)
    pp, ps, pb = field(plain), field(sur), field(base)
    out = {
        "sk_err_learned": rel_sk_error(ss, sp), "sk_err_linear": rel_sk_error(sb, sp),
        "phi_err_learned": float((ps - pp).double().norm() / (pp - pp.mean()).double().norm()),
        "phi_err_linear": float((pb - pp).double().norm() / (pp - pp.mean()).double().norm()),
        "mass_err_learned": abs(float(ps.double().mean() - pp.double().mean())),
    }
    for s in (plain, sur, base):
        s.close()
    return out


def new_network(shape, params=None, norm=None, train=False, seed=0):
    """A network with given or fresh parameters (fresh: q2 = 0, so the
    correction starts at exactly zero and the macro step at L_K)."""
    net = FNO(shape, train=train)
    net.set_params(init_params(seed, out_scale=0.0) if params is None else params)
    if norm is not None:
        net.set_norm(norm)
    return net
