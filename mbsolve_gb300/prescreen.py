"""Surrogate prescreening of parameter sweeps.

A sweep space of 6-level media (the random-Hermitian 6-level family of the
6-level benchmark, scaled down) driven by one sech pulse. Each point has
six medium parameters and three pulse parameters:

    log10 carrier density      22 .. 24     (1/m^3)
    carrier dipole scale       0.5 .. 2     (the transition at the carrier)
    level detuning             -0.1 .. 0.1  (levels scaled by 1 + x)
    log10 scattering scale     -1 .. 1
    log10 dephasing scale      -1 .. 1
    other dipoles scale        0 .. 2       (the four other transitions)
    pulse amplitude            1e6 .. 3e7 V/m (log-uniform)
    pulse FWHM                 0.5 .. 1.5 ps
    pulse centre               1.5 .. 3 ps

The off-diagonal Hamiltonian terms are the base structure's, at a tenth
of their size: Lindblad dephasing acts in the bare level basis, so larger
couplings make it pump the medium out of its ground state within the
window (the medium would then radiate without a pulse).

The batched solver (ensemble, one launch sequence for all runs) gives the
probe field at the output facet; mbg_fno_envelope demodulates it at the
carrier into the transmitted envelope, sampled at S points over the
window. The surrogate (surrogate.FNO) learns envelope-in + parameters ->
envelope-out; sweeps then run on the surrogate and the solver judges its
error on the points it is asked about.

Network inputs per sample point s (F = 9 features): the input envelope
divided by its peak, the six medium parameters scaled to [-1, 1], the
log-amplitude scaled to [-1, 1], and s / S. The target is the transmitted
envelope divided by the input peak.
"""
import math
import time

import numpy as np
import torch

from . import ensemble as ens_mod
from . import lib as mb
from . import setups
from . import surrogate
from . import surrogate_kernels as K

PARAM_NAMES = ["log_density", "dipole_scale", "detuning", "log_scattering",
               "log_dephasing", "other_dipoles", "amplitude", "fwhm", "centre"]
COUPLING = 0.1
RANGES = {
    "log_density": (22.0, 24.0),
    "dipole_scale": (0.5, 2.0),
    "detuning": (-0.1, 0.1),
    "log_scattering": (-1.0, 1.0),
    "log_dephasing": (-1.0, 1.0),
    "other_dipoles": (0.0, 2.0),
    "amplitude": (1e6, 3e7),
    "fwhm": (0.5e-12, 1.5e-12),
    "centre": (1.5e-12, 3.0e-12),
}
MEDIUM = PARAM_NAMES[:6]
NUM_FEATURES = 9


class SweepSpace:
    """Base 6-level structure (seeded) and the grid every run uses."""

    def __init__(self, seed=0, num_gridpoints=224, length=50e-6,
                 window=8e-12, samples=1024, record_every=4):
        self.seed = seed
        self.n_x = num_gridpoints
        self.length = length
        self.window = window
        self.samples = samples
        self.record_every = record_every
        self._base(seed)
        dx = length / (num_gridpoints - 1)
        self.dt = 0.5 * dx * math.sqrt(mb.MU0 * mb.EPS0)
        self.n_t = int(round(window / self.dt))
        self.t_end = setups._courant_endtime(num_gridpoints, length, self.n_t)

    def _base(self, seed):
        """Levels uniform in 0-50 meV, couplings 1 % of that scale, five
        dipoles of 1e-29-5e-29 C m, rates log-uniform in 1e9-1e12 1/s; the
        carrier is the dipole-coupled transition in 3-8 THz with the
        largest dipole. Seeds without one, or with two levels closer than
        4 meV (which the couplings would mix strongly), are skipped.
        Scattering only goes down (from level n into m < n), so that the
        medium at rest stays at rest: it absorbs and re-emits the pulse but
        does not radiate by itself."""
        N = 6
        P = N * (N - 1) // 2
        pairs = [(i, j) for j in range(N) for i in range(j)]  # column-major upper
        s = seed
        while True:
            rng = np.random.default_rng(s)
            lv = np.sort(rng.uniform(0, 50e-3, size=N))
            hoff = (rng.normal(size=P) + 1j * rng.normal(size=P)) * 0.01 * 50e-3
            doff = np.zeros(P, dtype=complex)
            nz = rng.choice(P, size=5, replace=False)
            doff[nz] = rng.uniform(1e-29, 5e-29, size=5) * \
                np.exp(1j * rng.uniform(0, 2 * math.pi, size=5))
            scat = np.exp(rng.uniform(math.log(1e9), math.log(1e12), size=(N, N)))
            scat = np.triu(scat, 1)     # scat[m][n]: from n into m < n
            deph = np.exp(rng.uniform(math.log(1e9), math.log(1e12), size=P))
            best = None
            for q in nz:
                i, j = pairs[q]
                f = abs(lv[j] - lv[i]) * mb.E0 / (2 * math.pi * mb.HBAR)
                if 3e12 <= f <= 8e12 and (best is None or abs(doff[q]) > abs(doff[best[0]])):
                    best = (q, f)
            if best is not None and np.diff(lv).min() >= 4e-3:
                break
            s += 1000
        self.base_seed = s
        self.levels_ev, self.hoff_ev, self.doff = lv, hoff, doff
        self.scat, self.deph = scat, deph
        self.f0 = best[1]
        self.carrier = int(best[0])

    # ------------------------------------------------------------ points
    def sample(self, n, seed):
        """n points drawn uniformly (log-uniform amplitude)."""
        rng = np.random.default_rng(seed)
        p = {}
        for k in PARAM_NAMES:
            lo, hi = RANGES[k]
            if k == "amplitude":
                p[k] = np.exp(rng.uniform(math.log(lo), math.log(hi), size=n))
            else:
                p[k] = rng.uniform(lo, hi, size=n)
        return p

    def run(self, p, i):
        """(device, scenario) of point i."""
        N = 6
        det = 1.0 + p["detuning"][i]
        H = mb.qm_operator(list(self.levels_ev * det * mb.E0),
                           list(self.hoff_ev * COUPLING * mb.E0))
        u = mb.qm_operator([0.0] * N, list(self.dipoles(p, i)))
        relax = mb.qm_lindblad_relaxation(
            (self.scat * 10 ** p["log_scattering"][i]).tolist(),
            list(self.deph * 10 ** p["log_dephasing"][i]))
        qm = mb.qm_description(10 ** p["log_density"][i], H, u, relax)
        ar = setups._material("AR_sweep", qm)
        dev = mb.device("sweep")
        dev.add_region(mb.region("Active region", ar, 0.0, self.length))
        sce = mb.scenario("sweep", self.n_x, self.t_end,
                          mb.ic_density_const(self.ground_state(p, i)),
                          mb.ic_field_const(0.0), mb.ic_field_const(0.0))
        beta = 2.0 * math.acosh(2.0) / p["fwhm"][i]
        sce.add_source(mb.sech_pulse("pulse", 0.0, mb.source.hard_source,
                                     p["amplitude"][i], self.f0,
                                     beta * p["centre"][i], beta))
        sce.add_record(mb.record("e", self.record_every * self.dt, self.length))
        return dev, sce

    def dipoles(self, p, i):
        """Dipole matrix elements (packed upper triangle) of point i."""
        d = self.doff * p["other_dipoles"][i]
        d[self.carrier] = self.doff[self.carrier] * p["dipole_scale"][i]
        return d

    def hamiltonian(self, p, i):
        """Hermitian 6 x 6 Hamiltonian of point i in eV."""
        N = 6
        H = np.diag(self.levels_ev * (1.0 + p["detuning"][i])).astype(complex)
        pairs = [(a, b) for b in range(N) for a in range(b)]
        for q, (a, b) in enumerate(pairs):
            H[a, b] = self.hoff_ev[q] * COUPLING
            H[b, a] = np.conj(H[a, b])
        return H

    def ground_state(self, p, i):
        """Density matrix of the lowest eigenstate of point i's Hamiltonian
        (the medium at rest), as a qm_operator."""
        N = 6
        w, v = np.linalg.eigh(self.hamiltonian(p, i))
        g = v[:, 0]
        rho = np.outer(g, np.conj(g))
        pairs = [(a, b) for b in range(N) for a in range(b)]
        return mb.qm_operator(list(np.real(np.diag(rho))),
                              [rho[a, b] for a, b in pairs])

    def times(self):
        return np.arange(self.samples) * (self.window / self.samples)

    def envelope_in(self, p):
        """[n, S] input envelopes A sech(beta (t - t_c))."""
        t = self.times()[None, :]
        beta = (2.0 * math.acosh(2.0) / p["fwhm"])[:, None]
        return p["amplitude"][:, None] / np.cosh(beta * (t - p["centre"][:, None]))

    def features(self, p, device="cuda"):
        """FP32 [n, S, F] network inputs."""
        n = len(p["amplitude"])
        env = self.envelope_in(p)
        X = np.zeros((n, self.samples, NUM_FEATURES), np.float32)
        X[..., 0] = env / p["amplitude"][:, None]
        for k, name in enumerate(MEDIUM):
            lo, hi = RANGES[name]
            X[..., 1 + k] = (2.0 * (p[name] - lo) / (hi - lo) - 1.0)[:, None]
        lo, hi = RANGES["amplitude"]
        X[..., 7] = (2.0 * (np.log(p["amplitude"]) - math.log(lo)) /
                     (math.log(hi) - math.log(lo)) - 1.0)[:, None]
        X[..., 8] = (np.arange(self.samples) / self.samples)[None, :]
        return torch.tensor(X, device=device)

    # ------------------------------------------------------------ solver
    def solve(self, p, solver="gpu-fdtd-6lvl-cvr-rodr-fp32", chunk=2048,
              device="cuda"):
        """Transmitted envelopes [n, S] (FP32, on the GPU, divided by the
        input peak) from the batched solver, and the solver's wall time
        (set-up, run, result copy and demodulation)."""
        n = len(p["amplitude"])
        out = torch.empty(n, self.samples, dtype=torch.float32, device=device)
        seconds = 0.0
        for c0 in range(0, n, chunk):
            c1 = min(n, c0 + chunk)
            mb.material.clear_library()
            t0 = time.perf_counter()
            runs = [self.run(p, i) for i in range(c0, c1)]
            e = ens_mod.ensemble(solver, runs)
            e.run()
            rows = None
            tr = []
            for r in range(c1 - c0):
                a = e.results(r)[0].as_array()[:, 0]
                rows = len(a) if rows is None else min(rows, len(a))
                tr.append(a)
            e.close()
            E = torch.tensor(np.stack([a[:rows] for a in tr]), dtype=torch.float64,
                             device=device)
            dtr = self.record_every * self.dt
            env = torch.empty(c1 - c0, self.samples, dtype=torch.float32, device=device)
            K.envelope(E, 0.0, dtr, self.f0, self.samples, 0.0,
                       self.window / self.samples, env)
            amp = torch.tensor(p["amplitude"][c0:c1], dtype=torch.float32, device=device)
            out[c0:c1] = env / amp[:, None]
            torch.cuda.synchronize()
            seconds += time.perf_counter() - t0
        return out, seconds


def train(net, X, Y, epochs=20, batch=64, lr=2e-3, seed=0, weight_decay=1e-4,
          log=None):
    """Adam with a cosine learning-rate decay; returns per-epoch mean losses."""
    n = X.shape[0] - X.shape[0] % batch
    g = torch.Generator(device="cpu").manual_seed(seed)
    steps = epochs * (n // batch)
    hist, k = [], 0
    for ep in range(epochs):
        perm = torch.randperm(X.shape[0], generator=g)[:n].to(X.device)
        Xs, Ys = X.index_select(0, perm), Y.index_select(0, perm)
        tot = torch.zeros(1, device=X.device)
        for i in range(0, n, batch):
            rate = lr * 0.5 * (1.0 + math.cos(math.pi * k / steps))
            tot += net.train_step(Xs[i:i + batch], Ys[i:i + batch], lr=rate,
                                  weight_decay=weight_decay)
            k += 1
        hist.append(tot.item() / (n // batch))
        if log:
            log("epoch %d loss %.3e" % (ep, hist[-1]))
    return hist


def predict(net, X, batch=4096):
    """Surrogate outputs [n, S] for inputs X (FP32 [n, S, F]), through the
    network's inference path (FNO.infer), `batch` points per call (4,096:
    each fused layer launch then gives every SM ~27 samples, against ~7 at
    1,024, and the launch's last wave costs ~0.3 % instead of ~4 %)."""
    out = torch.empty(X.shape[0], X.shape[1], dtype=torch.float32, device=X.device)
    for i in range(0, X.shape[0], batch):
        xb = X[i:i + batch]
        out[i:i + xb.shape[0]] = net.infer(xb)
    return out


def rel_errors(pred, truth):
    """Per-run relative L2 error of predicted envelopes."""
    num = torch.linalg.vector_norm(pred - truth, dim=1)
    den = torch.linalg.vector_norm(truth, dim=1).clamp_min(1e-12)
    return (num / den).cpu().numpy()


def transmission(env_out, env_in):
    """Transmitted energy fraction per run (envelopes normalised alike)."""
    return ((env_out.double() ** 2).sum(1) / (env_in.double() ** 2).sum(1)).cpu().numpy()


def delayed_input(space, X):
    """The no-medium prediction: the input envelope delayed by the
    vacuum transit time of the device."""
    shift = int(round(space.length * math.sqrt(mb.MU0 * mb.EPS0) /
                      (space.window / space.samples)))
    env = X[..., 0]
    out = torch.zeros_like(env)
    out[:, shift:] = env[:, :env.shape[1] - shift]
    return out


def pipeline(n_train=20000, n_sweep=10000, n_judge=None, shapes=None,
             epochs=30, batch=64, lr=2e-3, seed=0, absorb=None,
             solver="gpu-fdtd-6lvl-cvr-rodr-fp32", log=None, infer_batch=4096):
    """Generate training runs with the solver, train the surrogate on the
    GPU, sweep n_sweep new points with it (infer_batch points per inference
    call) and judge it with the solver on n_judge of them (all by
    default). The prescreen question is "which
points transmit less than `absorb` of the pulse energy" (default: the
solver's lower quartile on the judged points). Returns a report dict."""
    def say(msg):
        if log:
            log(msg)
    shapes = shapes or surrogate.Shapes(F=NUM_FEATURES)
    space = SweepSpace(samples=shapes.S)
    rep = dict(space=dict(f0_hz=space.f0, levels_mev=list(np.round(space.levels_ev * 1e3, 3)),
                          n_x=space.n_x, n_t=space.n_t, length_m=space.length,
                          window_s=space.window, samples=space.samples,
                          base_seed=space.base_seed),
               network=dict(S=shapes.S, W=shapes.W, Mo=shapes.Mo, L=shapes.L,
                            F=shapes.F, Hq=shapes.Hq,
                            params=shapes.num_params(), dtype="bf16 products, fp32 accumulate"),
               solver=solver)
    p_tr = space.sample(n_train, seed=seed + 1)
    Y_tr, t_gen = space.solve(p_tr, solver=solver)
    X_tr = space.features(p_tr)
    rep["generate"] = dict(runs=n_train, seconds=t_gen, runs_per_s=n_train / t_gen)
    say("generated %d runs in %.1f s" % (n_train, t_gen))

    net = surrogate.FNO(shapes, seed=seed)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    hist = train(net, X_tr, Y_tr, epochs=epochs, batch=batch, lr=lr, seed=seed,
                 log=say)
    torch.cuda.synchronize()
    t_train = time.perf_counter() - t0
    rep["train"] = dict(epochs=epochs, batch=batch, steps=epochs * (n_train // batch),
                        seconds=t_train, loss_first=hist[0], loss_last=hist[-1])

    p_sw = space.sample(n_sweep, seed=seed + 2)
    X_sw = space.features(p_sw)
    # warm-up: the same calls (the inference buffers of each chunk size are
    # allocated once, outside the timed sweep)
    predict(net, X_sw, batch=infer_batch)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    pred = predict(net, X_sw, batch=infer_batch)
    torch.cuda.synchronize()
    t_sur = time.perf_counter() - t0
    nj = n_sweep if n_judge is None else min(n_judge, n_sweep)
    pj = {k: v[:nj] for k, v in p_sw.items()}
    truth, t_sol = space.solve(pj, solver=solver)
    err = rel_errors(pred[:nj], truth)
    err_vac = rel_errors(delayed_input(space, X_sw[:nj]), truth)
    mean_out = Y_tr.mean(0, keepdim=True).expand(nj, -1)
    err_mean = rel_errors(mean_out, truth)
    env_in = X_sw[:nj, :, 0]
    tr_true = transmission(truth, env_in)
    tr_pred = transmission(pred[:nj], env_in)
    if absorb is None:
        absorb = float(np.quantile(tr_true, 0.25))
    cls_true, cls_pred = tr_true < absorb, tr_pred < absorb
    tp = int((cls_true & cls_pred).sum())
    rep["sweep"] = dict(
        points=n_sweep, infer_batch=infer_batch, surrogate_seconds=t_sur,
        surrogate_runs_per_s=n_sweep / t_sur,
        judged=nj, solver_seconds=t_sol, solver_runs_per_s=nj / t_sol,
        speedup=(n_sweep / t_sur) / (nj / t_sol))
    rep["error"] = dict(
        metric="relative L2 error of the transmitted envelope per run, surrogate vs solver",
        median=float(np.median(err)), p90=float(np.quantile(err, 0.9)),
        mean=float(err.mean()),
        baseline_delayed_input_median=float(np.median(err_vac)),
        baseline_training_mean_median=float(np.median(err_mean)))
    rep["prescreen"] = dict(
        criterion="transmitted energy fraction < %.4g" % absorb,
        transmission_quantiles_solver=[float(x) for x in np.quantile(tr_true, [0, 0.1, 0.25, 0.5, 0.75, 0.9, 1])],
        positives_true=int(cls_true.sum()),
        accuracy=float((cls_true == cls_pred).mean()),
        precision=tp / max(1, int(cls_pred.sum())),
        recall=tp / max(1, int(cls_true.sum())))
    rep["status"] = K.status()
    say("sweep: surrogate %.0f runs/s, solver %.0f runs/s, median error %.3g"
        % (rep["sweep"]["surrogate_runs_per_s"], rep["sweep"]["solver_runs_per_s"],
           rep["error"]["median"]))
    return rep, net


def main(argv=None):
    import argparse
    import json
    ap = argparse.ArgumentParser(description="surrogate prescreening pipeline")
    ap.add_argument("--train", type=int, default=20000)
    ap.add_argument("--sweep", type=int, default=10000)
    ap.add_argument("--judge", type=int, default=None)
    ap.add_argument("--epochs", type=int, default=30)
    ap.add_argument("--samples", type=int, default=1024)
    ap.add_argument("--width", type=int, default=64)
    ap.add_argument("--modes", type=int, default=32)
    ap.add_argument("--layers", type=int, default=4)
    ap.add_argument("--out", default=None, help="write the report (JSON) here")
    ap.add_argument("--save", default=None, help="save the trained weights (.npy)")
    a = ap.parse_args(argv)
    sh = surrogate.Shapes(S=a.samples, W=a.width, Mo=a.modes, L=a.layers,
                          F=NUM_FEATURES)
    rep, net = pipeline(a.train, a.sweep, a.judge, sh, epochs=a.epochs,
                        log=lambda m: print(m, flush=True))
    s = json.dumps(rep, indent=1)
    print(s)
    if a.out:
        with open(a.out, "w") as f:
            f.write(s + "\n")
    if a.save:
        np.save(a.save, net.theta.cpu().numpy())


if __name__ == "__main__":
    main()
