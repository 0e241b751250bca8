"""Learned spectral multiplier for Fourier-accelerated Landau gauge fixing.

Method (no counterpart in the reference; written for this library):

* Fourier-accelerated steepest descent (Davies et al., Phys. Rev. D 37 (1988)
  1581) updates g <- exp(-F^-1[m(p) F[Delta]]/V) g with the fixed multiplier
  m(p) = alpha p2max/phat^2(p). In the linear regime a mode of the gauge
  condition Delta contracts as Delta(p) -> (1 - m(p) lambda(p)) Delta(p); the
  effective rate lambda depends on the configuration (beta) and on how far
  the fixing has got (theta).
* Training data: on HMC-generated SU(3) configurations with random gauge
  transforms, descent runs to theta < 1e-12; at the start of every decade of
  theta a search over a two-parameter multiplier family
  m(p) = alpha p2max/p^2 high^w(p) (step size, and a factor on the
  shortest-wavelength modes, fading in from p2max/4 to p2max) runs each member on a copy of g under
  the solver's own fallback policy until theta has dropped tenfold and keeps
  the cheapest (steps plus fallback sweeps). Its log multiplier at a set of momenta is the target for the
  features x = (log phat^2 - log p2max, 5 (beta - 6), (log10 theta + 7)/5).
  The network amortises the search: one inference per step instead of
  twenty trial runs per decade. (mesh_landau_fa_probe, the per-momentum response, is
  kept as a diagnostic: a residual-weighted response is not a safe per-mode
  multiplier, as stiffer modes in a bin get over-stepped.)
* Network: 3 -> 64 -> 64 -> 1 tanh MLP (FP32 weights), trained on the GPU by
  the library's own forward/backward/Adam kernels (mesh_mlp_train); used with
  BF16 inference (mesh_landau_fa_set_mlp) to rebuild the multiplier table
  before every step. Overrelaxation is the fallback whenever a step fails to
  lower theta (mesh_landau_fa_run).

`python -m mesh_gb300.landau_learn train` regenerates the committed weights
(landau_mlp_su3.npz, and the same parameters as raw FP32 in landau_mlp_su3.f32
for C and C++ callers) on a GPU; `... compare` prints the comparison.
"""
from __future__ import annotations

import argparse
import json
import os
import time

import numpy as np

from . import (ALGEBRA, F32, F64, GROUP, Context, Field, GaugeField, Grid, Hmc, Landau, LandauFA, Lattice,
               gauge_transform, make_deltas, mlp_forward, mlp_init, mlp_train, reunitize)

HERE = os.path.dirname(os.path.abspath(__file__))
WEIGHTS = os.path.join(HERE, "landau_mlp_su3.npz")
WIDTH = 64
PLAIN_ALPHA = 0.08  # Davies et al.'s step size; the largest stable one found


def features(log_p2_rel, beta, theta):
    return np.stack([np.asarray(log_p2_rel, dtype=np.float64), np.full_like(log_p2_rel, 5.0 * (beta - 6.0)),
                     np.full_like(log_p2_rel, (np.log10(max(theta, 1e-30)) + 7.0) / 5.0)], 1)


def hmc_configs(ctx, L, betas, seeds, therm, per_chain, spacing, eps=0.5, substeps=20):
    """SU(3) configurations from independent mixed-precision HMC chains (one
    per (beta, seed)), yielded one at a time as (beta, FP32 host array in the
    reference layout); only the current chain is held."""
    grid = Grid([L] * 4)
    d = make_deltas("2mn", eps, substeps)
    for beta, seed in zip(betas, seeds):
        h = Hmc(ctx, 3, F32, grid, seed=int(seed))
        h.randomize_gauge_field()
        h.run(float(beta), d, therm, use_graph=True)
        for _ in range(per_chain):
            if spacing:
                h.run(float(beta), d, spacing, use_graph=True)
            yield float(beta), h.U.export()
        h.close()


def prepared_links(ctx, U_host, transform_seed):
    """FP64 links on the device: reunitised in FP64 (from FP32 HMC output)
    and given a Haar-random gauge transform."""
    L = U_host.shape[1]
    dims = [int(round(L ** 0.25))] * 4
    U = GaugeField(ctx, 3, F64, Grid(dims)).import_(U_host.astype(np.float64))
    reunitize(U)
    reunitize(U)
    h = Lattice(ctx, 3, F64, Grid(dims)).random(int(transform_seed))
    gauge_transform(U, h)
    return U


# multiplier family searched during data collection:
#   m(p) = alpha p2max/p^2 * high^w(p),  w = clip(log(4 p^2 / p2max) / log 4, 0, 1):
# `high` scales the shortest-wavelength modes (p^2 = p2max) and fades out at
# p2max/4; high = 1 is the plain multiplier. A survey on thermalised 16^4
# configurations found the steps that fail to lower theta (and so cost an
# overrelaxation fallback) driven by those modes: damping them cut the cost
# of plain descent by a quarter, while raising the longest-wavelength modes
# multiplied the fallbacks.
ALPHAS = (0.06, 0.08, 0.1)
HIGHS = (1.0, 0.5, 0.35, 0.2)
TABLE_N = 256


def family_mult(alpha, high, p2, p2min, p2max, low=1.0):
    """alpha p2max/p^2 high^w_hi low^w_lo: w_hi ramps (in log p^2) from 0 at
    p2max/4 to 1 at p2max, w_lo from 1 at p2min to 0 at 4 p2min"""
    w_hi = np.clip(np.log(4.0 * p2 / p2max) / np.log(4.0), 0.0, 1.0)
    w_lo = np.clip(np.log(4.0 * p2min / p2) / np.log(4.0), 0.0, 1.0)
    return alpha * p2max / p2 * high ** w_hi * low ** w_lo


def family_table(alpha, high, p2min, p2max, n=TABLE_N, low=1.0):
    lo, hi = np.log(p2min) - 1e-3, np.log(p2max) + 1e-3
    p2 = np.exp(np.linspace(lo, hi, n))
    return np.log(family_mult(alpha, high, p2, p2min, p2max, low)).astype(np.float32), lo, hi


def survey(ctx, L, seeds, members, therm=100, transform_seed=5, max_iter=5000, accept="theta"):
    """Fixed multipliers family_mult(alpha, high, low) over configurations:
    {member: [(steps, fallbacks, cost), ...]} with cost = steps + 11 x
    fallbacks; a member that does not converge in max_iter steps costs 99999.
    Steps are accepted on `accept` ("theta" or "functional")."""
    res = {m: [] for m in members}
    for beta, Uh in hmc_configs(ctx, L, [6.0] * len(seeds), seeds, therm, 1, 0):
        for m in members:
            U = prepared_links(ctx, Uh, transform_seed)
            fa = LandauFA(U)
            fa.set_accept(accept == "functional")
            p2min, p2max = fa.p2range()
            fa.set_table(*family_table(m[0], m[1], p2min, p2max, low=m[2]))
            g = Lattice(ctx, 3, F64, U.grid).set_unit()
            it, fb, th = fa.run(g, tol=1e-12, max_iter=max_iter)
            res[m].append((it, fb, it + 11 * fb) if th < 1e-12 else (it, fb, 99999))
            fa.close()
    return res


def collect(ctx, U, beta, tol=1e-12, nbins=24, max_steps=400, omega=1.7, or_sweeps=10, sample=None,
            accept="theta", alphas=None, highs=None):
    """Samples along a data-collection run, one set per decade of theta. At
    the start of a decade every member (alpha, high) of the multiplier
    family runs on a copy of g under the solver's own policy (a step that
    does not lower theta is undone and replaced by `or_sweeps`
    overrelaxation sweeps) until theta has dropped tenfold; its cost is
    steps + (or_sweeps + 1) x fallbacks (a step and a sweep cost about the
    same). The cheapest member's log multiplier at `nbins` momenta is the
    target for the features (log p^2/p2max, beta, theta) at the decade's
    start and middle; g advances to that member's result. With `sample` (a
    set of decade numbers, 0 = the first) only those decades are searched;
    the others advance with the plain multiplier. Steps are accepted on
    `accept` ("theta" or "functional"; under the functional test no step
    falls back and the cost is the number of steps). Rows: (3 features,
    target)."""
    alphas = ALPHAS if alphas is None else alphas
    highs = HIGHS if highs is None else highs
    fa = LandauFA(U)
    fa.set_accept(accept == "functional")
    p2min, p2max = fa.p2range()
    g = Lattice(U.ctx, 3, F64, U.grid).set_unit()
    trial = Lattice(U.ctx, 3, F64, U.grid)
    best_g = Lattice(U.ctx, 3, F64, U.grid)
    rows = []
    centers = np.exp(np.linspace(np.log(p2min), np.log(p2max), nbins))
    lnd = Landau(U)
    lnd.g = g
    cost_total = 0
    collect.log = []
    decade = -1
    while True:
        th = fa.theta(g)
        if th < tol:
            break
        target = max(th / 10.0, tol)
        decade += 1
        if sample is not None and decade not in sample:
            fa.set_plain(PLAIN_ALPHA)
            it, fb, _ = fa.run(g, tol=target, max_iter=20 * max_steps, omega=omega, or_sweeps=or_sweeps)
            cost_total += it + (or_sweeps + 1) * fb
            continue
        best = None
        plain_cost = None
        for a in alphas:
            for b in highs:
                fa.set_table(*family_table(a, b, p2min, p2max))
                trial.copy_from(g)
                it, fb, th_end = fa.run(trial, tol=target, max_iter=max_steps, omega=omega, or_sweeps=or_sweeps)
                if not th_end < target:
                    continue
                cost = it + (or_sweeps + 1) * fb
                if a == PLAIN_ALPHA and b == 1.0:
                    plain_cost = cost
                if best is None or cost < best[0]:
                    best = (cost, a, b)
                    best_g.copy_from(trial)
        collect.log.append({"theta": th, "plain_cost": plain_cost,
                            "best": None if best is None else {"cost": best[0], "alpha": best[1], "high": best[2]}})
        if best is None:
            it, _ = lnd.overrelax(omega, tol=target, max_sweeps=20 * max_steps, check_every=10)
            cost_total += it
            continue
        cost, a, b = best
        tgt = np.log(family_mult(a, b, centers, p2min, p2max))
        for t in (th, th / np.sqrt(10.0)):
            rows.append(np.column_stack([features(np.log(centers) - np.log(p2max), beta, t), tgt]))
        g.copy_from(best_g)
        cost_total += cost
    fa.close()
    collect.last_cost = cost_total
    return np.concatenate(rows) if rows else np.zeros((0, 4))


def train(ctx, data, epochs=200, batch=1024, lr=2e-3, seed=0):
    x = data[:, :3].astype(np.float32)
    t = data[:, 3].astype(np.float32)
    p0 = mlp_init(WIDTH, seed)
    params, losses = mlp_train(ctx, x, t, p0, WIDTH, epochs=epochs, batch=batch, lr=lr, seed=seed)
    return params, losses


def solve(ctx, U, method, params=None, beta=6.0, tol=1e-12, max_iter=20000, omega=1.7, accept="functional",
          member=None):
    """Fix U to Landau gauge from g = 1 with `method` in {"or", "plain",
    "learned", "fixed"} ("fixed": the family member (alpha, high) given as
    `member`);
    Fourier-accelerated steps are accepted on `accept` ("theta" or
    "functional"); returns dict(seconds, iterations, fallbacks, theta, functional)."""
    import torch

    g = Lattice(U.ctx, 3, F64, U.grid).set_unit()
    fa = None
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    if method == "or":
        L = Landau(U)
        L.g = g
        it, th = L.overrelax(omega, tol=tol, max_sweeps=max_iter, check_every=10)
        fb = 0
    else:
        fa = LandauFA(U)
        fa.set_accept(accept == "functional")
        if method == "plain":
            fa.set_plain(PLAIN_ALPHA)
        elif method == "fixed":
            p2min, p2max = fa.p2range()
            fa.set_table(*family_table(member[0], member[1], p2min, p2max))
        else:
            fa.set_mlp(params, WIDTH, beta, bf16=True)
        it, fb, th = fa.run(g, tol=tol, max_iter=max_iter, omega=omega, or_sweeps=10)
    torch.cuda.synchronize()
    secs = time.perf_counter() - t0
    L = Landau(U)
    L.g = g
    res = {"method": method, "seconds": secs, "iterations": it, "fallbacks": fb, "theta": th, "functional": L()}
    if fa is not None:
        fa.close()
    return res


def load_weights(path=WEIGHTS):
    z = np.load(path)
    return z["params"].astype(np.float32), float(z["gamma"])


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("mode", choices=["train", "compare", "survey"])
    ap.add_argument("--configs", type=int, default=256)
    ap.add_argument("--chains", type=int, default=16)
    ap.add_argument("--L", type=int, default=24)
    ap.add_argument("--therm", type=int, default=100)
    ap.add_argument("--spacing", type=int, default=5)
    ap.add_argument("--eval-L", type=int, default=32)
    ap.add_argument("--eval-configs", type=int, default=32)
    ap.add_argument("--eval-therm", type=int, default=200)
    ap.add_argument("--out", default=WEIGHTS)
    ap.add_argument("--seed0", type=int, default=11, help="survey: HMC seed of the first configuration")
    ap.add_argument("--json", default=None)
    ap.add_argument("--sample-decades", type=int, default=0,
                    help="search this many random decades per configuration (0: every decade)")
    ap.add_argument("--accept", choices=["theta", "functional"], default="functional",
                    help="acceptance test of the Fourier-accelerated steps (survey, train, compare)")
    ap.add_argument("--alphas", default=None, help="train: comma-separated step sizes of the family search")
    ap.add_argument("--highs", default=None, help="train: comma-separated high-mode factors of the family search")
    ap.add_argument("--fixed", default="0.08,0.6", help="compare: the fixed family member alpha,high")
    ap.add_argument("--weights", default=WEIGHTS, help="compare: the network to evaluate")
    ap.add_argument("--methods", default="or,plain,fixed,learned", help="compare: solvers to run")
    args = ap.parse_args()
    ctx = Context(0)
    if args.mode == "survey":
        alphas = tuple(float(x) for x in args.alphas.split(",")) if args.alphas else (0.06, 0.08, 0.1, 0.12)
        highs = tuple(float(x) for x in args.highs.split(",")) if args.highs else (1.0, 0.6, 0.35)
        lows = (1.0,) if args.alphas else (1.0, 2.0)
        members = [(a, h, b) for a in alphas for h in highs for b in lows]
        seeds = list(range(args.seed0, args.seed0 + args.configs))
        res = survey(ctx, args.L, seeds, members, therm=args.therm, accept=args.accept)
        for c, m, v in sorted((float(np.mean([x[2] for x in v])), m, v) for m, v in res.items()):
            print(json.dumps({"alpha": m[0], "high": m[1], "low": m[2], "mean_cost": c, "cost": [x[2] for x in v],
                              "fallbacks": [x[1] for x in v]}))
        return
    if args.mode == "train":
        t0 = time.time()
        rng = np.random.default_rng(99)
        betas = rng.uniform(5.8, 6.2, args.chains)
        per_chain = max(1, args.configs // args.chains)
        cfgs = hmc_configs(ctx, args.L, betas, np.arange(1000, 1000 + args.chains), args.therm, per_chain,
                           args.spacing)
        data = []
        ncfg = 0
        for k, (beta, Uh) in enumerate(cfgs):
            ncfg += 1
            U = prepared_links(ctx, Uh, transform_seed=5000 + k)
            sample = None
            if args.sample_decades:
                sample = set(int(x) for x in rng.choice(12, args.sample_decades, replace=False))
            alphas = tuple(float(x) for x in args.alphas.split(",")) if args.alphas else None
            highs = tuple(float(x) for x in args.highs.split(",")) if args.highs else None
            data.append(collect(ctx, U, beta, sample=sample, accept=args.accept, alphas=alphas, highs=highs))
            print(json.dumps({"config": k, "beta": beta, "collect_cost": collect.last_cost, "decades": collect.log,
                              "rows": int(len(data[-1]))}), flush=True)
        data = np.concatenate(data)
        t_collect = time.time() - t0
        params, losses = train(ctx, data)
        np.savez(args.out, params=params, gamma=1.0, width=WIDTH, samples=len(data),
                 final_loss=float(losses[-1]), first_loss=float(losses[0]), configs=ncfg, lattice=args.L,
                 betas=betas, accept=args.accept)
        # the same parameters as raw little-endian FP32 for C and C++ callers
        np.asarray(params, dtype="<f4").tofile(os.path.splitext(args.out)[0] + ".f32")
        print(json.dumps({"samples": int(len(data)), "final_loss": float(losses[-1]),
                          "first_loss": float(losses[0]), "target_variance": float(np.var(data[:, 3])),
                          "t_generate_and_collect_s": t_collect, "configs": ncfg}))
    else:
        params, gamma = load_weights(args.weights)
        seeds = np.arange(1, args.eval_configs + 1)
        cfgs = hmc_configs(ctx, args.eval_L, [6.0] * len(seeds), seeds, args.eval_therm, 1, 0)
        rows = []
        fixed = tuple(float(x) for x in args.fixed.split(","))
        methods = tuple(m for m in args.methods.split(",") if m)
        for k, (beta, Uh) in enumerate(cfgs):
            for method in methods:
                U = prepared_links(ctx, Uh, transform_seed=5)
                r = solve(ctx, U, method, params, beta, accept=args.accept, member=fixed)
                r["config"] = k
                r["cost"] = r["iterations"] + 11 * r["fallbacks"] if method != "or" else r["iterations"]
                rows.append(r)
                print(json.dumps(r), flush=True)
        summ = {"accept": args.accept, "fixed_member": fixed, "weights": os.path.basename(args.weights)}
        for m in methods:
            rs = [r for r in rows if r["method"] == m]
            summ[m] = {"mean_seconds": float(np.mean([r["seconds"] for r in rs])),
                       "mean_iterations": float(np.mean([r["iterations"] for r in rs])),
                       "total_fallbacks": int(sum(r["fallbacks"] for r in rs)),
                       "total_cost": int(sum(r["cost"] for r in rs)),
                       "max_theta": float(max(r["theta"] for r in rs))}
        for m in ("or", "plain", "fixed"):
            if m in summ and "learned" in summ:
                summ[f"speedup_learned_vs_{m}"] = summ[m]["mean_seconds"] / summ["learned"]["mean_seconds"]
        print(json.dumps(summ))
        if args.json:
            with open(args.json, "w") as fh:
                json.dump({"rows": rows, "summary": summ}, fh)


if __name__ == "__main__":
    main()
