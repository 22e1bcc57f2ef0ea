"""Learned per-cell LU-SGS relaxation: training data from the solver's own
convergence histories, training on the device, and the driver that runs a
case with the network and falls back to the plain update.

Data.  A case is advanced with the plain LU-SGS update while the library
keeps each step's previous increment.  At snapshot iterations n the 12
features of every cell are taken (cfd_case_features); then, from the saved
state, the solver runs K steps once per candidate relaxation factor applied
to every cell (1.0, 1.2, 1.4, 1.6: the range in which a uniform factor stays
stable on these cases), and the target of every cell is the candidate after
which the case's L2 density residual is smallest (per-cell outcomes proved
too noisy: half the cells pointed at 1.0, half at 1.6, and a network fitted
to them mixed neighbouring factors into an unstable field).  The run then continues from the saved
state with the plain update.  Targets are stored as the network's raw
outputs (the inverse of omega = 1 + 0.6 sigmoid(o0)); the CFL output is trained
towards a multiplier of 1, since on these viscous cases the time step barely
moves the LU-SGS diagonal (measured: CFL x0.5 and x2 change the iteration
count by under 5%).

Pooling.  The network predicts a factor for every cell; the update applies the
mesh mean of the predictions (spread 0), optionally widened to mean +- spread.
Measured on held-out cases: per-cell factors (no bound) stall where factors
near 1.0 and 1.6 meet; spread 0.2 / 0.1 / 0 need 0.93 / 0.87 / 0.78 of the
plain iterations, the last matching the best uniform factor found by search.

Run.  run_to_drop() attaches the network after a few plain steps and watches
the L2 density residual every `chunk` steps; if it rises above `fallback`
times the best value seen, the network is detached and the run continues
with the plain update (the reference's method), which also decides the
converged state.
"""
from __future__ import annotations

import time
from dataclasses import dataclass

import numpy as np

from . import abi, configs, meshgen


OMEGA_SPAN = 0.6  # omega = 1 + OMEGA_SPAN * sigmoid(o0), as in k_mlp.cu


@dataclass
class CaseSpec:
    """One training or evaluation case: a cylinder mixed mesh (the recipe of
    the C2 workload at a smaller size) and a flow."""

    nbody: int = 64
    nlayer: int = 12
    seed: int = 7
    mach: float = 0.2
    aoa: float = 0.0
    re: float = 40.0
    cfl: float = 50.0
    flow: str = "laminar"
    dr1: float = 1e-2
    growth: float = 1.1
    rfar: float = 15.0

    def mesh(self) -> abi.Mesh:
        m = meshgen.mixed_mesh(configs.cylinder(self.nbody), nlayer=self.nlayer, dr1=self.dr1, growth=self.growth,
                               rfar=self.rfar, seed=self.seed, density=1.0, grade=0.82)
        import tempfile
        from pathlib import Path
        p = Path(tempfile.mkdtemp()) / "m.grd"
        meshgen.write_grd(p, m)
        return abi.Mesh.load_grd(p, -1, -2)

    def case(self, mesh: abi.Mesh, precision: int = abi.PREC_FP64) -> abi.Case:
        c = abi.Case([mesh], [dict(mach=self.mach, aoa_deg=self.aoa, reynolds=self.re)],
                     abi.FLOW_LAMINAR if self.flow == "laminar" else abi.FLOW_EULER, abi.ADV_LUSGS, precision,
                     cfl=self.cfl)
        c.init_freestream()
        return c


def sweep_specs(n: int, seed: int = 0, family: str = "small") -> list[CaseSpec]:
    """Seeded Mach / AoA / Reynolds sweep of cylinder cases.

    family "small": 5-10k cells (10-15 layers, outer radius 15 D); "c2": the
    C2 recipe (first spacing 5e-3 D, growth 1.05, outer radius 30 D) with
    24-40 layers and 96-160 body points, 15-40k cells."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        common = dict(seed=int(rng.integers(1, 1 << 20)), mach=float(rng.uniform(0.15, 0.4)),
                      aoa=float(rng.uniform(-4, 10)), re=float(rng.choice([20.0, 40.0, 100.0])), cfl=50.0)
        if family == "c2":
            out.append(CaseSpec(nbody=int(rng.choice([96, 128, 160])), nlayer=int(rng.integers(24, 41)),
                                dr1=5e-3, growth=1.05, rfar=30.0, **common))
        else:
            out.append(CaseSpec(nbody=int(rng.choice([48, 64, 80])), nlayer=int(rng.integers(10, 16)), **common))
    return out


def constant_net(omega: float) -> abi.Mlp:
    """A network whose output is the same relaxation factor in every cell."""
    m = abi.Mlp(0)
    p, norm = m.params()
    p[:] = 0
    q = min(max((omega - 1.0) / OMEGA_SPAN, 1e-4), 1 - 1e-4)
    p[-2] = np.log(q / (1.0 - q))
    m.set_params(p, norm)
    return m


def generate(specs, snapshots=(40, 80, 160, 320, 640, 1000), K: int = 30,
             candidates=(1.0, 1.1, 1.2, 1.3, 1.4, 1.5, 1.6),
             precision: int = abi.PREC_FP64):
    """(X, T, M) numpy arrays: features, raw-output targets and weights.

    At every snapshot the state is saved and advanced K steps once per
    candidate relaxation factor (applied uniformly); every cell's target is
    the candidate after which the case's L2 density residual is smallest.
    The CFL output is trained towards 1 (raw 0)."""
    import torch

    nets = {om: constant_net(om) for om in candidates if om != 1.0}
    Xs, Ts, Ms = [], [], []
    for spec in specs:
        mesh = spec.mesh()
        case = spec.case(mesh, precision)
        abi.case_track(case, True)
        nc = case.ncell
        feat = torch.empty(nc * abi.MLP_INPUTS, dtype=torch.float32, device="cuda")
        it = 0
        for n in snapshots:
            if n > it:
                case.step_graph(n - it)
            it = n
            case.sync()
            abi.case_features(case, feat.data_ptr())
            case.sync()
            X = feat.view(nc, abi.MLP_INPUTS).cpu().numpy().copy()
            U = case.get("U")
            score = np.empty(len(candidates))
            for j, om in enumerate(candidates):
                case.put("U", U)
                abi.case_set_mlp(case, nets.get(om))
                case.step(K)
                try:
                    score[j] = case.norm("L2_R_RHO")
                except abi.CfdError:
                    score[j] = np.inf
            abi.case_set_mlp(case, None)
            case.put("U", U)
            best = np.full(nc, candidates[int(np.argmin(score))])
            q = np.clip((best - 1.0) / OMEGA_SPAN, 1e-3, 1 - 1e-3)
            t0 = np.log(q / (1 - q))
            ok = np.isfinite(X).all(1)
            Xs.append(X[ok])
            Ts.append(np.stack([t0, np.zeros_like(t0)], 1)[ok].astype(np.float32))
            Ms.append(np.ones((ok.sum(), 2), np.float32))
        case.close()
    return np.concatenate(Xs), np.concatenate(Ts), np.concatenate(Ms)


def fit(X, T, M, steps: int = 3000, batch: int = 4096, lr: float = 2e-3, seed: int = 1):
    """Train a fresh network on the device; returns (mlp, loss history)."""
    import torch

    mlp = abi.Mlp(seed)
    mean = X.mean(0)
    std = X.std(0)
    p, _ = mlp.params()
    mlp.set_params(p, np.concatenate([mean, 1.0 / np.maximum(std, 1e-6)]).astype(np.float32))
    dx = torch.tensor(X, dtype=torch.float32, device="cuda")
    dt = torch.tensor(T, dtype=torch.float32, device="cuda")
    dm = torch.tensor(M, dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    hist = mlp.train(dx.data_ptr(), dt.data_ptr(), dm.data_ptr(), len(X), steps, min(batch, len(X)), lr, seed)
    return mlp, hist


@dataclass
class RunResult:
    reached: bool
    iterations: int
    seconds: float
    history: list
    fell_back: bool


def run_to_drop(case: abi.Case, target: float, max_iters: int, mlp: abi.Mlp | None = None, apply_cfl: bool = False,
                chunk: int = 25, warm: int = 20, fallback: float = 10.0, spread: float = 0.0,
                max_seconds: float | None = None, switch_at: float | None = None,
                switch_to: int | None = None, detach_at_switch: bool = False) -> RunResult:
    """Iterate until the L2 density residual falls by `target` (relative to iteration 1).

    switch_at / switch_to: once the residual has fallen by switch_at, or has
    fallen by less than 5% over the last 1000 iterations, the case switches to
    the precision form switch_to (cfd_set_precision), e.g. from the binary32
    form, whose residual stalls near 1e-4, to the mixed form.  detach_at_switch:
    the learned relaxation only runs until the switch."""
    lusgs = case.advance == abi.ADV_LUSGS
    if lusgs:
        abi.case_track(case, True)
    elif mlp is not None:
        raise ValueError("the learned relaxation needs the LU-SGS integrator")
    case.step_graph(1)
    r0 = case.norm("L2_R_RHO")
    it, best, fell = 1, 1.0, False
    hist = [(1, 1.0)]
    attached = False
    saved = None
    save_every = 500  # iterations between restart points (each is a device-to-host copy of the state)
    t0 = time.perf_counter()
    while it < max_iters and (max_seconds is None or time.perf_counter() - t0 < max_seconds):
        if mlp is not None and not attached and not fell and it >= warm:
            abi.case_set_mlp(case, mlp, apply_cfl, spread)
            attached = True
        if attached and (saved is None or it - saved[0] >= save_every):
            saved = (it, case.get("U"))  # restart point should a learned chunk fail
        try:
            case.step_graph(chunk)
            it += chunk
            r = case.norm("L2_R_RHO") / r0
        except abi.CfdError:
            if not attached:
                raise
            r = float("nan")
        hist.append((it, r))
        if attached and not (r <= fallback * best):
            abi.case_set_mlp(case, None)  # the plain update from here on
            attached, fell = False, True
            if not r == r:  # non-finite state: restart the plain update from the saved one
                it = saved[0]
                case.put("U", saved[1])
                continue
        best = min(best, r) if r == r else best
        if switch_at is not None and switch_to is not None:
            # switch at the given fall, or earlier if the residual has stopped
            # falling (less than 5% over the last 1000 iterations)
            back = [h for h in hist if h[0] <= it - 1000]
            stalled = bool(back) and not (r < 0.95 * back[-1][1])
            if r <= switch_at or stalled:
                case.set_precision(switch_to)
                switch_at = None
                if detach_at_switch and attached:
                    abi.case_set_mlp(case, None)  # the plain update in the second form
                    attached = False
                    mlp = None
        if r <= target:
            break
    el = time.perf_counter() - t0
    if attached:
        abi.case_set_mlp(case, None)
    return RunResult(bool(hist[-1][1] <= target), it, el, hist, fell)


WEIGHTS = __import__("pathlib").Path(__file__).resolve().parent / "relax_mlp.npz"


def save(mlp: abi.Mlp, path=WEIGHTS, **meta):
    p, n = mlp.params()
    np.savez(path, params=p, norm=n, **{k: np.asarray(v) for k, v in meta.items()})


def load(path=WEIGHTS) -> abi.Mlp | None:
    """The committed trained network, or None when the file is absent."""
    import pathlib
    if not pathlib.Path(path).exists():
        return None
    z = np.load(path)
    m = abi.Mlp(0)
    m.set_params(z["params"], z["norm"])
    return m


def main(argv=None):
    """Train the relaxation network on the seeded sweep and save it (needs a GPU)."""
    import argparse
    ap = argparse.ArgumentParser(description=main.__doc__)
    ap.add_argument("--cases", type=int, default=8, help="training cases of the seeded sweep")
    ap.add_argument("--family", default="c2", choices=["small", "c2"])
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3000)
    ap.add_argument("--out", default=str(WEIGHTS))
    a = ap.parse_args(argv)
    X, T, M = generate(sweep_specs(a.cases, seed=a.seed, family=a.family))
    mlp, hist = fit(X, T, M, steps=a.steps)
    save(mlp, a.out, samples=len(X), cases=a.cases, seed=a.seed, steps=a.steps, final_loss=float(hist[-1]),
         family=a.family)
    print(f"trained on {len(X)} cells of {a.cases} cases; loss {hist[0]:.4g} -> {hist[-1]:.4g}; saved {a.out}")


if __name__ == "__main__":
    main()
