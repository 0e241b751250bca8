"""Learned spectral multiplier for Fourier-accelerated Landau gauge fixing.

Method (no counterpart in the reference; written for this library):

* Fourier-accelerated steepest descent (Davies et al., Phys. Rev. D 37 (1988)
  1581) updates g <- exp(-F^-1[m(p) F[Delta]]/V) g with the fixed multiplier
  m(p) = alpha p2max/phat^2(p). In the linear regime a mode of the gauge
  condition Delta contracts as Delta(p) -> (1 - m(p) lambda(p)) Delta(p); the
  effective rate lambda depends on the configuration (beta) and on how far
  the fixing has got (theta).
* Training data: on HMC-generated SU(3) configurations with random gauge
  transforms, plain descent runs to theta < 1e-12 and is probed along the way
  (mesh_landau_fa_probe): a trial step with a small known multiplier gives
  lambda per bin of log phat^2. Each bin is a sample
  x = (log phat^2 - log p2max, 5 (beta - 6), (log10 theta + 7)/5),
  target = log(gamma / lambda), gamma a damping factor.
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


NONLINEAR_THETA = 1e-2  # above: indefinite Hessian, steps chosen by trial
ALPHAS = (0.01, 0.02, 0.04, 0.06, 0.08, 0.12)


def measured_table(pr, p2min, p2max, gamma, n=256):
    """log multiplier gamma/lambda on the table grid from a probe, the
    contraction rate clipped to [0.02, 20] (p^2/p2max) and interpolated in
    log p^2; None when the probe has no usable bin"""
    ok = (pr["count"] > 0) & np.isfinite(pr["lambda"])
    if not np.any(ok):
        return None
    p2 = pr["p2"][ok]
    lam = np.clip(pr["lambda"][ok], 0.02 * p2 / p2max, 20.0 * p2 / p2max)
    lo, hi = np.log(p2min) - 1e-3, np.log(p2max) + 1e-3
    grid = np.linspace(lo, hi, n)
    return np.interp(grid, np.log(p2), np.log(gamma / lam)).astype(np.float32), lo, hi


def collect(ctx, U, beta, gamma=0.5, probe_alpha=0.02, nbins=32, every=3, tol=1e-12, max_iter=600):
    """Samples along a data-collection run. theta > 1e-2: the best plain step
    size of a trial line search, target log(alpha* p2max/p^2) for every bin;
    theta <= 1e-2: probed contraction rates, target log(gamma/lambda), and the
    run is driven by the measured multiplier (refreshed every `every` steps).
    Rows: (3 features, target, regime) with regime 0 nonlinear, 1 linear."""
    fa = LandauFA(U)
    fa.mult_mode = 0
    p2min, p2max = fa.p2range()
    g = Lattice(U.ctx, 3, F64, U.grid).set_unit()
    rows = []
    centers = np.exp(np.linspace(np.log(p2min), np.log(p2max), nbins))
    for it in range(max_iter):
        th = fa.theta(g)
        if th < tol:
            break
        if th > NONLINEAR_THETA:
            res = [(fa.trial(g, a)[1], a) for a in ALPHAS]
            th_best, a_best = min(res)
            f = features(np.log(centers) - np.log(p2max), beta, th)
            rows.append(np.column_stack([f, np.log(a_best * p2max / centers), np.zeros(nbins)]))
            fa.set_plain(a_best)
            fa.mult_mode = 0
            fa.step(g)
            continue
        if it % every == 0 or fa.mult_mode != 1:
            pr = fa.probe(g, probe_alpha, nbins)
            ok = (pr["count"] > 0) & np.isfinite(pr["lambda"])
            lam = np.clip(pr["lambda"][ok], 0.02 * pr["p2"][ok] / p2max, 20.0 * pr["p2"][ok] / p2max)
            f = features(np.log(pr["p2"][ok]) - np.log(p2max), beta, pr["theta"])
            rows.append(np.column_stack([f, np.log(lam), np.ones(int(ok.sum()))]))
            tab = measured_table(pr, p2min, p2max, gamma)
            if tab is not None:
                fa.set_table(*tab)
                fa.mult_mode = 1
        before, after = fa.trial(g)
        if after < before:
            fa.step(g)
        else:
            # step rejected: a few overrelaxation sweeps (the run's fallback)
            Lnd = Landau(U)
            Lnd.g = g
            Lnd.overrelax(1.7, tol=0.0, max_sweeps=5, check_every=5)
            fa.mult_mode = 0
    fa.close()
    collect.last_iterations = it
    return np.concatenate(rows) if rows else np.zeros((0, 5))


def train(ctx, data, gamma, epochs=150, batch=2048, lr=2e-3, seed=0):
    """targets: nonlinear rows keep log(alpha* p2max/p^2); linear rows
    become log(gamma/lambda)"""
    x = data[:, :3].astype(np.float32)
    lin = data[:, 4] > 0.5
    t = np.where(lin, np.log(gamma) - data[:, 3], data[:, 3]).astype(np.float32)
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
        # damping: pick gamma on four training configurations
        best = None
        for gamma in (0.3, 0.5, 0.7, 1.0):
            params, losses = train(ctx, data, gamma)
            tot = 0.0
            for k in range(4):
                U = prepared_links(ctx, cfgs[k][1], transform_seed=7000 + k)
                tot += solve(ctx, U, "learned", params, cfgs[k][0], max_iter=3000)["seconds"]
            if best is None or tot < best[0]:
                best = (tot, gamma, params, losses)
        _, gamma, params, losses = best
        np.savez(args.out, params=params, gamma=gamma, width=WIDTH, samples=len(data),
                 final_loss=float(losses[-1]), configs=len(cfgs), lattice=args.L)
        print(json.dumps({"samples": int(len(data)), "gamma": gamma, "final_loss": float(losses[-1]),
                          "first_loss": float(losses[0]), "t_generate_s": t_gen, "t_collect_s": t_collect,
                          "configs": len(cfgs)}))
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
