"""Learned spectral multiplier for Fourier-accelerated Landau gauge fixing.

Method (no counterpart in the reference; written for this library):

* Fourier-accelerated steepest descent (Davies et al., Phys. Rev. D 37 (1988)
  1581) updates g <- exp(-F^-1[m(p) F[Delta]]/V) g with the fixed multiplier
  m(p) = alpha p2max/phat^2(p). In the linear regime a mode of the gauge
  condition Delta contracts as Delta(p) -> (1 - m(p) lambda(p)) Delta(p); the
  effective rate lambda depends on the configuration (beta) and on how far
  the fixing has got (theta).
* Training data: on HMC-generated SU(3) configurations with random gauge
  transforms, descent runs to theta < 1e-12; every few steps a trial line
  search (mesh_landau_fa_trial, g unchanged) over a two-parameter multiplier
  family m(p) = alpha p2max/p^2 max(1, boost 4 p2min/p^2) (step size and a
  boost of the slow long-wavelength modes) picks the member that lowers theta
  most. Its log multiplier at a set of momenta is the target for the
  features x = (log phat^2 - log p2max, 5 (beta - 6), (log10 theta + 7)/5).
  The network amortises the line search: one inference per step instead of
  a dozen trial steps. (mesh_landau_fa_probe, the per-momentum response, is
  kept as a diagnostic: a residual-weighted response is not a safe per-mode
  multiplier, as stiffer modes in a bin get over-stepped.)
* Network: 3 -> 64 -> 64 -> 1 tanh MLP (FP32 weights), trained on the GPU by
  the library's own forward/backward/Adam kernels (mesh_mlp_train); used with
  BF16 inference (mesh_landau_fa_set_mlp) to rebuild the multiplier table
  before every step. Overrelaxation is the fallback whenever a step fails to
  lower theta (mesh_landau_fa_run).

`python -m mesh_gb300.landau_learn train` regenerates the committed weights
(landau_mlp_su3.npz) on a GPU; `... compare` prints the comparison.
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
    per (beta, seed)), returned as FP64 host arrays in the reference layout
    together with their beta."""
    grid = Grid([L] * 4)
    d = make_deltas("2mn", eps, substeps)
    out = []
    for beta, seed in zip(betas, seeds):
        h = Hmc(ctx, 3, F32, grid, seed=int(seed))
        h.randomize_gauge_field()
        h.run(float(beta), d, therm, use_graph=True)
        for _ in range(per_chain):
            if spacing:
                h.run(float(beta), d, spacing, use_graph=True)
            out.append((float(beta), h.U.export().astype(np.float64)))
        h.close()
    return out


def prepared_links(ctx, U_host, transform_seed):
    """FP64 links on the device: reunitised in FP64 (from FP32 HMC output)
    and given a Haar-random gauge transform."""
    L = U_host.shape[1]
    dims = [int(round(L ** 0.25))] * 4
    U = GaugeField(ctx, 3, F64, Grid(dims)).import_(U_host)
    reunitize(U)
    reunitize(U)
    h = Lattice(ctx, 3, F64, Grid(dims)).random(int(transform_seed))
    gauge_transform(U, h)
    return U


# multiplier family searched per step during data collection:
#   m(p) = alpha * p2max/p^2 * max(1, boost * p2ref/p^2),  p2ref = 4 p2min
ALPHAS = (0.03, 0.05, 0.08, 0.11)
BOOSTS = (1.0, 2.0, 4.0)
TABLE_N = 256


def family_table(alpha, boost, p2min, p2max, n=TABLE_N):
    lo, hi = np.log(p2min) - 1e-3, np.log(p2max) + 1e-3
    lp = np.linspace(lo, hi, n)
    p2 = np.exp(lp)
    m = alpha * p2max / p2 * np.maximum(1.0, boost * 4.0 * p2min / p2)
    return np.log(m).astype(np.float32), lo, hi


def collect(ctx, U, beta, every=4, tol=1e-12, max_iter=1500, nbins=24):
    """Samples along a data-collection run: every `every` steps a trial line
    search over the multiplier family (alpha, boost) picks the member giving
    the lowest theta after one step; its log multiplier at `nbins` momenta is
    the target for features (log p^2/p2max, beta, theta). The run advances
    with that member, overrelaxation sweeps when a step fails to lower theta.
    Rows: (3 features, target)."""
    fa = LandauFA(U)
    p2min, p2max = fa.p2range()
    g = Lattice(U.ctx, 3, F64, U.grid).set_unit()
    rows = []
    centers = np.exp(np.linspace(np.log(p2min), np.log(p2max), nbins))
    lnd = Landau(U)
    lnd.g = g
    it = 0
    for it in range(max_iter):
        th = fa.theta(g)
        if th < tol:
            break
        if it % every == 0:
            best = None
            for a in ALPHAS:
                for b in BOOSTS:
                    fa.set_table(*family_table(a, b, p2min, p2max))
                    after = fa.trial(g)[1]
                    if best is None or after < best[0]:
                        best = (after, a, b)
            _, a, b = best
            tab = family_table(a, b, p2min, p2max)
            fa.set_table(*tab)
            tgt = np.log(a * p2max / centers * np.maximum(1.0, b * 4.0 * p2min / centers))
            rows.append(np.column_stack([features(np.log(centers) - np.log(p2max), beta, th), tgt]))
        before, after = fa.trial(g)
        if after < before:
            fa.step(g)
        else:
            lnd.overrelax(1.7, tol=0.0, max_sweeps=10, check_every=10)
    fa.close()
    collect.last_iterations = it
    return np.concatenate(rows) if rows else np.zeros((0, 4))


def train(ctx, data, epochs=200, batch=1024, lr=2e-3, seed=0):
    x = data[:, :3].astype(np.float32)
    t = data[:, 3].astype(np.float32)
    p0 = mlp_init(WIDTH, seed)
    params, losses = mlp_train(ctx, x, t, p0, WIDTH, epochs=epochs, batch=batch, lr=lr, seed=seed)
    return params, losses


def solve(ctx, U, method, params=None, beta=6.0, tol=1e-12, max_iter=20000, omega=1.7):
    """Fix U to Landau gauge from g = 1 with `method` in {"or", "plain", "learned"};
    returns dict(seconds, iterations, fallbacks, theta, functional)."""
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
        if method == "plain":
            fa.set_plain(PLAIN_ALPHA)
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
    ap.add_argument("mode", choices=["train", "compare"])
    ap.add_argument("--configs", type=int, default=256)
    ap.add_argument("--chains", type=int, default=16)
    ap.add_argument("--L", type=int, default=24)
    ap.add_argument("--therm", type=int, default=100)
    ap.add_argument("--spacing", type=int, default=5)
    ap.add_argument("--eval-L", type=int, default=32)
    ap.add_argument("--eval-configs", type=int, default=32)
    ap.add_argument("--eval-therm", type=int, default=200)
    ap.add_argument("--out", default=WEIGHTS)
    ap.add_argument("--json", default=None)
    args = ap.parse_args()
    ctx = Context(0)
    if args.mode == "train":
        t0 = time.time()
        rng = np.random.default_rng(99)
        betas = rng.uniform(5.8, 6.2, args.chains)
        per_chain = max(1, args.configs // args.chains)
        cfgs = hmc_configs(ctx, args.L, betas, np.arange(1000, 1000 + args.chains), args.therm, per_chain,
                           args.spacing)
        t_gen = time.time() - t0
        data = []
        for k, (beta, Uh) in enumerate(cfgs):
            U = prepared_links(ctx, Uh, transform_seed=5000 + k)
            data.append(collect(ctx, U, beta))
            print(json.dumps({"config": k, "beta": beta, "collect_iterations": collect.last_iterations,
                              "rows": int(len(data[-1]))}), flush=True)
        data = np.concatenate(data)
        t_collect = time.time() - t0 - t_gen
        params, losses = train(ctx, data)
        np.savez(args.out, params=params, gamma=1.0, width=WIDTH, samples=len(data),
                 final_loss=float(losses[-1]), first_loss=float(losses[0]), configs=len(cfgs), lattice=args.L,
                 betas=betas)
        print(json.dumps({"samples": int(len(data)), "final_loss": float(losses[-1]),
                          "first_loss": float(losses[0]), "target_variance": float(np.var(data[:, 3])),
                          "t_generate_s": t_gen, "t_collect_s": t_collect, "configs": len(cfgs)}))
    else:
        params, gamma = load_weights()
        seeds = np.arange(1, args.eval_configs + 1)
        cfgs = hmc_configs(ctx, args.eval_L, [6.0] * len(seeds), seeds, args.eval_therm, 1, 0)
        rows = []
        for k, (beta, Uh) in enumerate(cfgs):
            for method in ("or", "plain", "learned"):
                U = prepared_links(ctx, Uh, transform_seed=5)
                r = solve(ctx, U, method, params, beta)
                r["config"] = k
                rows.append(r)
                print(json.dumps(r), flush=True)
        summ = {}
        for m in ("or", "plain", "learned"):
            rs = [r for r in rows if r["method"] == m]
            summ[m] = {"mean_seconds": float(np.mean([r["seconds"] for r in rs])),
                       "mean_iterations": float(np.mean([r["iterations"] for r in rs])),
                       "total_fallbacks": int(sum(r["fallbacks"] for r in rs)),
                       "max_theta": float(max(r["theta"] for r in rs))}
        summ["speedup_learned_vs_or"] = summ["or"]["mean_seconds"] / summ["learned"]["mean_seconds"]
        summ["speedup_learned_vs_plain"] = summ["plain"]["mean_seconds"] / summ["learned"]["mean_seconds"]
        print(json.dumps(summ))
        if args.json:
            with open(args.json, "w") as fh:
                json.dump({"rows": rows, "summary": summ}, fh)


if __name__ == "__main__":
    main()
