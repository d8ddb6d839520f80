#!/usr/bin/env python
"""HPS build+solve benchmark on one GB300.

Workload ``poisson`` (default): 2D variable-coefficient problem on
[-1,1]^2, L = d_xx + d_yy + c(x,y), c = 1 + 0.5 * sum of 4 Gaussian bumps
(seeded centres in [-0.8,0.8]^2, width 0.2); uniform quadtree L=7 (16384
leaves), p=16, q=14, DtN; 64 right-hand sides, each a seeded sum of 8
Gaussian sources (width 0.1) with Dirichlet data b_j (x^2 - y^2).  FP32
build + FP64 refinement against the plain FP64 path.

Workload ``helmholtz`` (--workload helmholtz): 2D Helmholtz scattering with
ItI maps, Delta u + k^2 (1 + q) u = f, k = 40, q = 0.5 * sum of 20 seeded
Gaussian bumps (width 0.05), scattered-field source f = -k^2 q u_in for a
plane wave u_in at a seeded angle, zero incoming impedance data, eta = k;
uniform quadtree L=8 (65536 leaves), p=16, q=14, one right-hand side.
complex64 build + complex128 refinement against the plain complex128 path.

Workload ``c1``: the same operator form at L=3, p=8, q=6 (64 leaves), the
manufactured solution u = sin(pi x) sin(pi y) (c = 1 + 0.5 * 4 seeded
bumps), plain FP64, boundary data u and x^2 - y^2: compared with the
reference's own output (tests/golden/c1_dtn2d_L3_p8.npz) and the oracle.

Workload ``c4``: 3D, [-1,1]^3, c = 1 + 0.3 * 6 seeded bumps, u = sin sin
sin, uniform octree L=3 (512 leaves), p=10, q=8: FP32 build + FP64
refinement against the plain FP64 GPU path.

Workload ``c5``: adaptive octree meshing of f = Laplacian of
arctan(50(|x - x0| - 0.7)), x0 = (-0.05,)*3, on [0,1]^3, p=10, q=8,
tol 1e-5 (L-infinity): meshing time of the plain criterion and with the
learned refinement proposal (trained first on other fronts), every accepted
leaf judged by the plain criterion; then the FP64 build + solve on the tree.

One step = build_solver + solve of all right-hand sides.
Metric: leaves/s = n_leaves / (t_build + t_solve).

  value : inputs already resident in HBM, result left in HBM.
  e2e   : through the public API with pinned host inputs; the host->device
          copies of coefficients/source/boundary data and the device->host
          copy of the solution (into a page-locked buffer the caller keeps,
          solve(..., out=buf)) are inside the timed region.

Accuracy: the mixed result is compared with the plain FP64 GPU path and,
for ``poisson``, with the FP64 CPU oracle run on the same inputs at the same
size (relative L2 and max-norm errors).

``cpu_baseline`` / ``--impl reference``: the CPU restatement of the
reference algorithm (the FP64 oracle; the reference's own JAX code cannot be
installed on these machines).  For ``poisson`` it is the level-batched oracle
(``oracle/hps_oracle_level.py``) on the full workload, on every host thread;
for ``helmholtz`` the per-leaf loop oracle on an L=4 sample.

Prints one JSON line (rank 0).
"""

from __future__ import annotations

import argparse
import json
import os
import subprocess
import tempfile
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

WORKLOADS = {
    "poisson": dict(name="2D var-coeff DtN, uniform quadtree", L=7, p=16, q=14, nsrc=64),
    "helmholtz": dict(name="2D Helmholtz scattering ItI k=40, uniform quadtree", L=8, p=16, q=14, nsrc=1, k=40.0),
    "c1": dict(name="2D var-coeff DtN, manufactured sin(pi x) sin(pi y), plain FP64", L=3, p=8, q=6, nsrc=1),
    "c4": dict(name="3D var-coeff DtN, manufactured sin sin sin, uniform octree", L=3, p=10, q=8, nsrc=1),
    "c5": dict(name="3D adaptive octree wavefront arctan(50(|x-x0|-0.7)), meshing with and without the MLP",
               L=None, p=10, q=8, nsrc=1, tol=1e-5),
}
WORKLOAD = WORKLOADS["poisson"]


# ---------------------------------------------------------------------------
# workload
# ---------------------------------------------------------------------------


def bump_centres(seed=0):
    return np.random.default_rng(seed).uniform(-0.8, 0.8, (4, 2))


def coefficient_c(x, z):
    r2 = ((x[..., None, :] - z) ** 2).sum(-1)
    return 1.0 + 0.5 * np.exp(-r2 / 0.2 ** 2).sum(-1)


def source_params(nsrc, seed=1):
    rng = np.random.default_rng(seed)
    a = rng.uniform(-1, 1, (nsrc, 8))
    zs = rng.uniform(-0.8, 0.8, (nsrc, 8, 2))
    b = rng.uniform(-1, 1, nsrc)
    return a, zs, b


def make_inputs(L, p, q, nsrc, device):
    """Domain, coefficient arrays and sources, generated on `device`."""
    import torch

    import jaxhps_gb300 as hps

    root = hps.DiscretizationNode2D(-1.0, 1.0, -1.0, 1.0)
    dom = hps.Domain(p=p, q=q, root=root, L=L)
    x = torch.as_tensor(dom.interior_points, device=device)
    z = torch.as_tensor(bump_centres(), device=device)
    c = 1.0 + 0.5 * torch.exp(-((x[..., None, :] - z) ** 2).sum(-1) / 0.2 ** 2).sum(-1)
    a, zs, b = (torch.as_tensor(t, device=device) for t in source_params(nsrc))
    f = torch.empty(x.shape[:2] + (nsrc,), dtype=torch.float64, device=device)
    for j in range(nsrc):
        f[..., j] = (a[j] * torch.exp(-((x[..., None, :] - zs[j]) ** 2).sum(-1) / 0.1 ** 2)).sum(-1)
    bp = torch.as_tensor(dom.boundary_points, device=device)
    g = (bp[:, 0] ** 2 - bp[:, 1] ** 2)[:, None] * b[None, :]
    ones = torch.ones_like(c)
    return dom, dict(D_xx_coefficients=ones, D_yy_coefficients=ones, I_coefficients=c), f, g


def helmholtz_fields(x, k, seed=40):
    """(q, u_in) of the scattering workload at points x (..., 2), numpy."""
    rng = np.random.default_rng(seed)
    z = rng.uniform(-0.8, 0.8, (20, 2))
    qv = 0.5 * np.exp(-((x[..., None, :] - z) ** 2).sum(-1) / (2 * 0.05 ** 2)).sum(-1)
    th = rng.uniform(0, 2 * np.pi)
    uin = np.exp(1j * k * (x @ np.array([np.cos(th), np.sin(th)])))
    return qv, uin


def make_inputs_helmholtz(L, p, q, k, device):
    """Domain, coefficients (I = k^2 (1 + q)), source -k^2 q u_in and zero
    incoming impedance data, generated on `device`."""
    import torch

    import jaxhps_gb300 as hps

    root = hps.DiscretizationNode2D(-1.0, 1.0, -1.0, 1.0)
    dom = hps.Domain(p=p, q=q, root=root, L=L)
    x = torch.as_tensor(dom.interior_points, device=device)
    rng = np.random.default_rng(40)
    z = torch.as_tensor(rng.uniform(-0.8, 0.8, (20, 2)), device=device)
    th = rng.uniform(0, 2 * np.pi)
    qv = 0.5 * torch.exp(-((x[..., None, :] - z) ** 2).sum(-1) / (2 * 0.05 ** 2)).sum(-1)
    d = torch.tensor([np.cos(th), np.sin(th)], dtype=torch.float64, device=device)
    uin = torch.exp(1j * k * (x @ d))
    f = (-k ** 2 * qv * uin).unsqueeze(-1).contiguous()
    g = torch.zeros((dom.boundary_points.shape[0], 1), dtype=torch.complex128, device=device)
    ones = torch.ones_like(qv)
    return dom, dict(D_xx_coefficients=ones, D_yy_coefficients=ones, I_coefficients=k ** 2 * (1 + qv),
                     use_ItI=True, eta=k), f, g


# ---------------------------------------------------------------------------
# clocks
# ---------------------------------------------------------------------------

CLOCK_Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
           "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
           "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")


class ClockSampler:
    def __init__(self):
        self.proc = None
        self.path = Path(tempfile.gettempdir()) / f"jaxhps_gb300_clocks_{os.getpid()}.csv"

    def start(self):
        try:
            self.path.parent.mkdir(exist_ok=True)
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={CLOCK_Q}", "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=self.fh, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.fh.close()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.path.read_text().splitlines():
            parts = [t.strip() for t in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        load = [s for s in sm if mx and s > 0.5 * mx] or sm
        return {"sm_mhz": float(np.median(load)) if load else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------------------
# CPU oracle timing (bounded sample of the same workload)
# ---------------------------------------------------------------------------


def cpu_oracle_sample_helmholtz(L_sample=4, p=16, q=14, k=40.0):
    from oracle import hps_oracle as O

    root = (-1.0, 1.0, -1.0, 1.0)
    pts = O.leaf_points_2D(O.uniform_leaf_bounds_2D(root, L_sample), p)
    qv, uin = helmholtz_fields(pts, k)
    ones = np.ones_like(qv)
    t0 = time.perf_counter()
    pr = O.Problem2D(root, L_sample, p, q, {"D_xx": ones, "D_yy": ones, "I": k ** 2 * (1 + qv)}, -k ** 2 * qv * uin,
                     iti=True, eta=k).build()
    pr.solve(np.zeros(pr.boundary_points.shape[0], dtype=np.complex128))
    dt = time.perf_counter() - t0
    n = 4 ** L_sample
    return n / dt, dt, n


def host_inputs(L, p, q, nsrc):
    """The poisson workload's coefficient, sources and boundary data as NumPy
    arrays (generated with torch on the CPU, the same formulas as on the GPU)."""
    _, coeffs, f, g = make_inputs(L, p, q, nsrc, "cpu")
    return coeffs["I_coefficients"].numpy(), f.numpy(), g.numpy()


def oracle_poisson(c, f, g, L, p, q, threads=None):
    """Build + solve of the poisson workload by the level-batched FP64 oracle;
    returns (solution, seconds)."""
    from oracle import hps_oracle_level as OL

    ones = np.ones_like(c)
    t0 = time.perf_counter()
    pr = OL.LevelProblem2D((-1.0, 1.0, -1.0, 1.0), L, p, q, {"D_xx": ones, "D_yy": ones, "I": c}, f, threads=threads)
    pr.build()
    u = pr.solve(g)
    dt = time.perf_counter() - t0
    pr.close()
    return u, dt


def oracle_thread_speedup(L=5, p=16, q=14, nsrc=64):
    """Speed-up of the level-batched oracle on every host thread over one
    thread, on an L=5 instance of the poisson workload."""
    c, f, g = host_inputs(L, p, q, nsrc)
    _, t1 = oracle_poisson(c, f, g, L, p, q, threads=1)
    _, tn = oracle_poisson(c, f, g, L, p, q)
    return t1 / tn


def cpu_threads():
    try:
        return len(os.sched_getaffinity(0))
    except Exception:
        return os.cpu_count() or 1


# ---------------------------------------------------------------------------
# main
# ---------------------------------------------------------------------------


def max_over_ranks(x: float, device) -> float:
    """The largest x over the ranks of the default process group (x itself
    when there is none or it has one rank); every rank gets the result."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(x)
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def _cpu_sample_helmholtz(args):
    L_s = min(args.ref_L, 4)
    v, dt, n = cpu_oracle_sample_helmholtz(L_s)
    what = (f"complex128 NumPy/SciPy oracle (ItI), build+solve of the same problem at L={L_s} ({n} leaves, p=16, "
            f"q=14, 1 RHS); Python loops over leaves and merges, OpenBLAS threads inside each call")
    return v, dt, n, what


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    wl = WORKLOADS[args.workload]
    vals = []
    if args.workload in ("c4", "c5"):
        print(json.dumps({"impl": "reference", "unavailable": "the CPU oracle needs minutes per step at this size "
                          "(c4: --workload c4 --oracle times it once beside the GPU run)"}))
        return 0
    if args.workload == "c1":
        import jaxhps_gb300 as hps
        from oracle import hps_oracle as O

        L, p, q = wl["L"], wl["p"], wl["q"]
        dom = hps.Domain(p=p, q=q, root=hps.DiscretizationNode2D(-1.0, 1.0, -1.0, 1.0), L=L)
        c, f, g0, g1, _ = c1_inputs(dom)
        ones = np.ones_like(c)
        for i in range(args.warmup + args.steps):
            t0 = time.perf_counter()
            ref = O.Problem2D((-1.0, 1.0, -1.0, 1.0), L, p, q, {"D_xx": ones, "D_yy": ones, "I": c}, f).build()
            ref.solve(g0)
            ref.solve(g1)
            if i >= args.warmup:
                vals.append(4 ** L / (time.perf_counter() - t0))
        same, speedup = True, None
        sample = f"the full workload (L={L}, build + 2 solves) by the FP64 NumPy oracle, per-leaf loops"
    elif args.workload == "helmholtz":
        for i in range(args.warmup + args.steps):
            v, dt, n, sample = _cpu_sample_helmholtz(args)
            if i >= args.warmup:
                vals.append(v)
        same, speedup = False, None
    else:
        L, p, q, ns = args.L, wl["p"], wl["q"], wl["nsrc"]
        c, f, g = host_inputs(L, p, q, ns)
        for i in range(args.warmup + args.steps):
            _, dt = oracle_poisson(c, f, g, L, p, q)
            if i >= args.warmup:
                vals.append(4 ** L / dt)
        same = True
        speedup = oracle_thread_speedup(L=min(5, L), p=p, q=q, nsrc=ns)
        sample = (f"the full workload (L={L}, {4 ** L} leaves, p={p}, q={q}, {ns} RHS) per step: level-batched FP64 "
                  f"NumPy oracle (CPU restatement of the reference algorithm), LAPACK/BLAS batches on a thread pool "
                  f"(one BLAS thread each) for levels of many small problems and BLAS on every thread for the top "
                  f"merges; all threads run an L={min(5, L)} instance {speedup:.1f}x faster than one")
    value = float(np.mean(vals))
    line = {
        "impl": "reference", "metric": "build+solve leaves/s", "value": value, "unit": "leaves/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
        "dtype": "c128" if args.workload == "helmholtz" else "f64", "data": "synthetic",
        "config": {"workload": wl["name"], "L": args.L, "p": wl["p"], "q": wl["q"], "nsrc": wl["nsrc"]},
        "same_config": same,
        "cpu_baseline": {"value": value, "unit": "leaves/s", "cores": cpu_threads(), "kind": "port",
                         "sample": sample, "thread_speedup": speedup},
        "e2e": {"value": value, "unit": "leaves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "the reference's JAX package cannot be installed offline here; its algorithm is timed as the "
                "oracle port",
    }
    print(json.dumps(line))
    return 0


def _errs(a, b) -> dict:
    a, b = np.asarray(a), np.asarray(b)
    return {"rel_l2": float(np.linalg.norm((a - b).ravel()) / max(np.linalg.norm(b.ravel()), 1e-300)),
            "rel_linf": float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))}


def _time_steps(step, steps, warmup):
    """CUDA-event time of `steps` calls after `warmup` untimed ones, with
    clocks sampled during the timed region; returns (ms per step, clocks, last result)."""
    import torch

    out = None
    for _ in range(warmup):
        out = step()
    torch.cuda.synchronize()
    clocks = ClockSampler()
    clocks.start()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(steps):
        out = step()
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / steps, clocks.stop(), out


def _base_line(args, wl, metric, value, unit, ms, higher=True, dtype="f64", extra_config=None):
    cfg = {"workload": wl["name"], **{k: wl[k] for k in ("L", "p", "q", "nsrc") if wl.get(k) is not None},
           "parallelism": "single-gpu"}
    cfg.update(extra_config or {})
    return {"metric": metric, "value": value, "unit": unit, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms, "higher_is_better": higher, "scaling": "weak", "vs_baseline": None, "dtype": dtype,
            "data": "synthetic", "config": cfg}


def c1_inputs(dom):
    x = np.asarray(dom.interior_points)
    bp = np.asarray(dom.boundary_points)
    z = np.random.default_rng(0).uniform(-0.8, 0.8, (4, 2))
    c = 1.0 + 0.5 * np.exp(-((x[..., None, :] - z) ** 2).sum(-1) / 0.2 ** 2).sum(-1)
    u = np.sin(np.pi * x[..., 0]) * np.sin(np.pi * x[..., 1])
    f = (c - 2 * np.pi ** 2) * u
    g0 = np.sin(np.pi * bp[:, 0]) * np.sin(np.pi * bp[:, 1])
    g1 = bp[:, 0] ** 2 - bp[:, 1] ** 2
    return c, f, g0, g1, u


def run_c1(args):
    """c1: plain FP64 build + two solves, against the reference's own output."""
    import torch

    import jaxhps_gb300 as hps
    from jaxhps_gb300 import _native as nat
    from oracle import hps_oracle as O

    wl = WORKLOADS["c1"]
    torch.cuda.set_device(0)
    dev = torch.device("cuda", 0)
    L, p, q = wl["L"], wl["p"], wl["q"]
    dom = hps.Domain(p=p, q=q, root=hps.DiscretizationNode2D(-1.0, 1.0, -1.0, 1.0), L=L)
    c, f, g0, g1, u_ex = c1_inputs(dom)
    ones = np.ones_like(c)
    tc = {k: torch.as_tensor(v, device=dev) for k, v in (("c", c), ("f", f), ("g0", g0), ("g1", g1), ("one", ones))}
    pde = hps.PDEProblem(dom, source=tc["f"], D_xx_coefficients=tc["one"], D_yy_coefficients=tc["one"],
                         I_coefficients=tc["c"])

    def step():
        pde.reset()
        hps.build_solver(pde, precision="float64")
        return hps.solve(pde, tc["g0"], host_device=None), hps.solve(pde, tc["g1"], host_device=None)

    l0 = nat.launch_count()
    ms, clk, (u0, u1) = _time_steps(step, args.steps, args.warmup)
    launches = (nat.launch_count() - l0) // (args.steps + args.warmup)
    u0, u1 = u0.cpu().numpy(), u1.cpu().numpy()
    acc = {}
    fx_path = ROOT / "tests" / "golden" / "c1_dtn2d_L3_p8.npz"
    if fx_path.exists():
        with np.load(fx_path) as fx:
            acc["vs_reference_output"] = {"g=u": _errs(u0, fx["soln_0"]), "g=x^2-y^2": _errs(u1, fx["soln_1"])}
    t0 = time.perf_counter()
    ref = O.Problem2D((-1.0, 1.0, -1.0, 1.0), L, p, q, {"D_xx": ones, "D_yy": ones, "I": c}, f).build()
    r0, r1 = ref.solve(g0), ref.solve(g1)
    dt = time.perf_counter() - t0
    acc["vs_oracle"] = {"g=u": _errs(u0, r0), "g=x^2-y^2": _errs(u1, r1)}
    acc["discretization_error_vs_exact"] = float(np.abs(u0 - u_ex).max())
    # e2e through the public API from host buffers
    hf, hc, ho = (torch.as_tensor(a).pin_memory() for a in (f, c, ones))
    hg0, hg1 = torch.as_tensor(g0).pin_memory(), torch.as_tensor(g1).pin_memory()
    hu0, hu1 = torch.empty(u0.shape, dtype=torch.float64).pin_memory(), torch.empty(u1.shape, dtype=torch.float64).pin_memory()
    pde_h = hps.PDEProblem(dom, source=hf, D_xx_coefficients=ho, D_yy_coefficients=ho, I_coefficients=hc)

    def estep():
        pde_h.reset()
        hps.build_solver(pde_h, precision="float64")
        hps.solve(pde_h, hg0, out=hu0)
        hps.solve(pde_h, hg1, out=hu1)

    for _ in range(max(3, args.warmup)):
        estep()
    torch.cuda.synchronize()
    n_e = max(5, args.steps)
    te0 = time.perf_counter()
    for _ in range(n_e):
        estep()
    torch.cuda.synchronize()
    te = (time.perf_counter() - te0) / n_e
    n = dom.n_leaves
    line = _base_line(args, wl, "build+solve leaves/s", n / (ms / 1e3), "leaves/s", ms,
                      extra_config={"precision": "float64", "solves_per_step": 2, "l2": "small problem (L2-resident)"})
    line.update({
        **acc,
        "e2e": {"value": n / te, "unit": "leaves/s", "ms_per_step": te * 1e3,
                "h2d_bytes_per_step": int(8 * (f.size + 2 * c.size + g0.size + g1.size)),
                "d2h_bytes_per_step": int(8 * (u0.size + u1.size))},
        "gpu_launches": launches * args.steps,
        "cpu_baseline": {"value": n / dt, "unit": "leaves/s", "cores": cpu_threads(), "kind": "port",
                         "sample": f"the full workload (build + 2 solves) by the FP64 NumPy oracle, {dt * 1e3:.0f} ms"},
        "clocks": clk,
    })
    print(json.dumps(line))
    return 0


def c4_inputs(dom):
    x = np.asarray(dom.interior_points)
    bp = np.asarray(dom.boundary_points)
    z = np.random.default_rng(3).uniform(-0.8, 0.8, (6, 3))
    c = 1.0 + 0.3 * np.exp(-((x[..., None, :] - z) ** 2).sum(-1) / 0.2 ** 2).sum(-1)
    u = np.sin(np.pi * x[..., 0]) * np.sin(np.pi * x[..., 1]) * np.sin(np.pi * x[..., 2])
    f = (c - 3 * np.pi ** 2) * u
    g = np.sin(np.pi * bp[:, 0]) * np.sin(np.pi * bp[:, 1]) * np.sin(np.pi * bp[:, 2])
    return c, f, g, u


def run_c4(args):
    """c4: 3D uniform octree, mixed precision against the plain FP64 GPU path."""
    import torch

    import jaxhps_gb300 as hps
    from jaxhps_gb300 import _native as nat

    wl = WORKLOADS["c4"]
    torch.cuda.set_device(0)
    dev = torch.device("cuda", 0)
    L, p, q = wl["L"], wl["p"], wl["q"]
    dom = hps.Domain(p=p, q=q, root=hps.DiscretizationNode3D(-1.0, 1.0, -1.0, 1.0, -1.0, 1.0), L=L)
    c, f, g, u_ex = c4_inputs(dom)
    ones = np.ones_like(c)
    kw = {k: torch.as_tensor(v, device=dev) for k, v in (("D_xx_coefficients", ones), ("D_yy_coefficients", ones),
                                                          ("D_zz_coefficients", ones), ("I_coefficients", c))}
    ft, gt = torch.as_tensor(f, device=dev), torch.as_tensor(g, device=dev)

    def make_step(prec):
        pde = hps.PDEProblem(dom, source=ft, **kw)

        def step():
            pde.reset()
            hps.build_solver(pde, precision=prec)
            return hps.solve(pde, gt, host_device=None)
        return pde, step

    pde, step = make_step(args.precision)
    l0 = nat.launch_count()
    ms, clk, u = _time_steps(step, args.steps, args.warmup)
    launches = (nat.launch_count() - l0) // (args.steps + args.warmup)
    iters = len(pde._state.history) if getattr(pde, "_state", None) is not None else None
    u = u.cpu().numpy()
    del pde, step
    nat.release_workspace()
    torch.cuda.empty_cache()
    pde64, step64 = make_step("float64")
    ms64, _, u64 = _time_steps(step64, max(1, args.fp64_steps), 1)
    u64 = u64.cpu().numpy()
    del pde64, step64
    n = dom.n_leaves
    line = _base_line(args, wl, "build+solve leaves/s", n / (ms / 1e3), "leaves/s", ms,
                      dtype={"float64": "f64", "float32": "f32", "mixed": "f32+f64-refinement"}[args.precision],
                      extra_config={"precision": args.precision, "l2": "operators of several GB (larger than L2)"})
    line.update({
        "rel_err_vs_fp64": _errs(u, u64), "refinement_iterations": iters,
        "discretization_error_vs_exact": {"this_path": float(np.abs(u - u_ex).max()),
                                          "fp64_path": float(np.abs(u64 - u_ex).max())},
        "fp64_path": {"value": n / (ms64 / 1e3), "unit": "leaves/s", "ms_per_step": ms64,
                      "speedup_of_this_path": ms64 / ms},
        "gpu_launches": launches * args.steps, "clocks": clk,
    })
    if args.oracle:
        from oracle import hps_oracle as O

        t0 = time.perf_counter()
        ref = O.Problem3D((-1.0, 1.0, -1.0, 1.0, -1.0, 1.0), L, p, q,
                          {"D_xx": ones, "D_yy": ones, "D_zz": ones, "I": c}, f).build()
        ur = ref.solve(g)
        dt = time.perf_counter() - t0
        line["rel_err_vs_oracle"] = _errs(u, ur)
        line["fp64_path_vs_oracle"] = _errs(u64, ur)
        line["cpu_baseline"] = {"value": n / dt, "unit": "leaves/s", "cores": cpu_threads(), "kind": "port",
                                "sample": f"the full workload by the FP64 NumPy oracle, {dt:.1f} s"}
    print(json.dumps(line))
    return 0


def wavefront_f(x0=(-0.05, -0.05, -0.05), a=50.0, R=0.7):
    """f = Laplacian of arctan(a (|x - x0| - R)) in 3D, for NumPy or torch points."""
    def f(x):
        xp = np if isinstance(x, np.ndarray) else __import__("torch")
        r = xp.sqrt(((x[..., 0] - x0[0]) ** 2 + (x[..., 1] - x0[1]) ** 2 + (x[..., 2] - x0[2]) ** 2))
        s = a * (r - R)
        return -2 * a ** 2 * s / (1 + s ** 2) ** 2 + 2 * a / (1 + s ** 2) / r
    return f


def wavefront_u(x0=(-0.05, -0.05, -0.05), a=50.0, R=0.7):
    def u(x):
        x = np.asarray(x)
        return np.arctan(a * (np.sqrt(((x - np.asarray(x0)) ** 2).sum(-1)) - R))
    return u


def run_c5(args):
    """c5: adaptive meshing with the plain criterion and with the learned
    refinement proposal, then the FP64 build + solve on the plain tree."""
    import torch

    import jaxhps_gb300 as hps
    from jaxhps_gb300 import _adaptive_discretization_3D as ad
    from jaxhps_gb300 import refinement_mlp as rm
    from jaxhps_gb300._discretization_tree import get_all_leaves

    wl = WORKLOADS["c5"]
    torch.cuda.set_device(0)
    dev = torch.device("cuda", 0)
    p, q, tol = wl["p"], wl["q"], wl["tol"]
    f = wavefront_f()

    def mesh(prop, stats=None):
        root = hps.DiscretizationNode3D(0.0, 1.0, 0.0, 1.0, 0.0, 1.0)
        ad.generate_adaptive_mesh_level_restriction(root, f, tol, p, q, proposer=prop, stats=stats)
        return root

    # the proposer is trained on refine / keep labels of other fronts (untimed)
    t_tr = time.perf_counter()
    rec = rm.LabelRecorder(device=dev)
    rng = np.random.default_rng(11)
    for _ in range(args.train_fronts):
        # centres outside the unit cube, as the target's: f has a 1/|x - x0| term
        c0 = tuple(-rng.uniform(0.02, 0.3, 3))
        ff = wavefront_f(c0, rng.uniform(20.0, 80.0), rng.uniform(0.5, 1.0))
        root = hps.DiscretizationNode3D(0.0, 1.0, 0.0, 1.0, 0.0, 1.0)
        ad.generate_adaptive_mesh_level_restriction(root, ff, tol, p, q, proposer=rec)
    X, y = rec.dataset()
    net = rm.RefinementMLP(device=dev, seed=0)
    net.train(X, y, epochs=40, batch=256, lr=2e-3)
    t_tr = time.perf_counter() - t_tr
    prop = rm.RefinementProposer(net, threshold=args.threshold)

    res = {}
    for name, pr in (("plain", None), ("mlp", prop)):
        for _ in range(args.warmup):
            mesh(pr)
        torch.cuda.synchronize()
        runs = []
        for _ in range(args.steps):
            st = {}
            root = mesh(pr, st)
            runs.append(st)
        res[name] = (root, runs)
    plain_s = float(np.median([r["seconds"] for r in res["plain"][1]]))
    mlp_s = float(np.median([r["seconds"] for r in res["mlp"][1]]))
    gn = res["plain"][1][-1]["global_norm"]
    consts = ad._CheckConstants(p, dev)
    judged = {}
    for name, (root, _) in res.items():
        leaves = get_all_leaves(root)
        diff, ref, _ = ad.refinement_check(np.array([lf.bounds for lf in leaves]), f, consts, dev)
        judged[name] = bool(np.all(diff / np.maximum(gn, ref) < tol))

    def summary(runs):
        r = runs[-1]
        keys = ("rounds", "checked", "proposed", "leaves", "t_propose", "t_check", "t_edit")
        return {**{k: r[k] for k in keys}, "seconds_median": float(np.median([x["seconds"] for x in runs])),
                "rounds_detail": r["rounds_detail"]}

    # FP64 build + solve on the plain tree
    n_labels = int(X.shape[0])
    del rec, X, y, net, prop
    torch.cuda.empty_cache()
    root = res["plain"][0]
    dom = hps.Domain(p=p, q=q, root=root)
    x = np.asarray(dom.interior_points)
    ones = np.ones(x.shape[:2])
    src = f(x)
    pde = hps.PDEProblem(dom, source=src, D_xx_coefficients=ones, D_yy_coefficients=ones, D_zz_coefficients=ones)
    bl = dom.get_adaptive_boundary_data_lst(wavefront_u())
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    try:
        hps.build_solver(pde)
        u = hps.solve(pde, bl)
        torch.cuda.synchronize()
        t_bs = time.perf_counter() - t0
        err = float(np.abs(np.asarray(u) - wavefront_u()(x)).max())
    except torch.OutOfMemoryError as e:
        t_bs, err = None, f"not run: {str(e).splitlines()[0][:160]}"
    line = _base_line(args, wl, "adaptive meshing seconds (learned proposal)", mlp_s, "s", mlp_s * 1e3, higher=False,
                      extra_config={"tol": tol, "criterion": "L-infinity", "proposal_threshold": args.threshold,
                                    "l2": "meshing: f evaluated per round on the GPU"})
    line.update({
        "plain_meshing_seconds": plain_s, "speedup_of_proposal": plain_s / mlp_s,
        "plain": summary(res["plain"][1]), "mlp": summary(res["mlp"][1]),
        "every_leaf_passes_plain_criterion": judged,
        "training": {"fronts": args.train_fronts, "labels": n_labels, "seconds": t_tr},
        "build_solve_fp64": {"leaves": dom.n_leaves, "seconds": t_bs,
                             "leaves_per_s": dom.n_leaves / t_bs if t_bs else None, "max_error_vs_exact_u": err},
    })
    print(json.dumps(line))
    return 0


CLASS_NAMES = {1: "gemm (SIMT tiles, 3xTF32 tcgen05 kernel)", 2: "inverse (merge interfaces; leaf blocks off the "
                "tensor cores)", 3: "gather/scatter/assembly", 4: "residual_2d_kernel (FP64 residual)",
               5: "gemm_tma_kernel (TMA + tcgen05, N <= 64 products)", 6: "jx_df_kernel (FP32-pair residual update)",
               7: "inv_tc_kernel (leaf inverses, tensor memory)"}
BYTES_CLASSES = (3, 5, 6)

# DRAM traffic per launch (dram__bytes_read.sum + dram__bytes_write.sum) from
# the ncu capture summarised in profiles/traffic_poisson_L5_mixed.md (L = 5),
# scaled by the number of leaves to L = 7 (the leaf kernels' traffic grows in
# proportion), for the classes with one launch shape per step:
# (workload, L, class) -> bytes
NCU_TRAFFIC = {("poisson", 7, 4): 16 * 281.2e6, ("poisson", 7, 6): 16 * 268.2e6, ("poisson", 7, 7): 16 * 254.9e6}


def class_roofline(nat, c, v, step_ms, peaks, mhz, res_bytes, workload, L):
    """Roofline record of one kernel class from the live profiler's totals
    (summed CUDA-event ms, launches, algorithmic work)."""
    k_ms, k_n, k_work = v
    avg_ms = k_ms / max(k_n, 1)
    if c in BYTES_CLASSES or c == 4:
        per = res_bytes if c == 4 else k_work / max(k_n, 1)
        peak = peaks.get("hbm_gbs", 6800.0)
        achieved = per / (avg_ms / 1e3) / 1e9
        r = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
             "traffic": NCU_TRAFFIC.get((workload, L, c)), "kernel": CLASS_NAMES[c], "bytes_per_launch": per,
             "peak_source": "MEASURED_PEAKS.json hbm_gbs, of measured" if peaks else "fallback 6800 GB/s"}
        if c == 4:
            r["flops_per_launch"] = k_work / max(k_n, 1)
            r["fp64_tflops"] = k_work / (k_ms / 1e3) / 1e12
    else:
        peak = peaks.get("bf16_tflops", 1900.0)
        achieved = k_work / (k_ms / 1e3) / 1e12
        # FP32 / TF32 arithmetic: besides the bf16 tensor peak the contract
        # names, the FP32 FMA rate (152 SMs x 128 lanes x 2 flop x the sampled
        # SM clock) bounds the SIMT kernels
        fp32_peak = 152 * 128 * 2 * mhz * 1e6 / 1e12
        r = {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
             "traffic": NCU_TRAFFIC.get((workload, L, c)), "kernel": CLASS_NAMES[c],
             "flops_per_launch": k_work / max(k_n, 1),
             "peak_source": "MEASURED_PEAKS.json bf16_tflops (burst), of measured" if peaks else "fallback",
             "fp32_simt_peak_tflops": fp32_peak, "frac_of_fp32_simt": achieved / fp32_peak}
    r["avg_launch_ms"] = avg_ms
    r["launches_in_timed_region"] = k_n
    r["share_of_step"] = k_ms / step_ms
    return r


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="mixed", choices=["float64", "float32", "mixed"])
    ap.add_argument("--fp64-steps", dest="fp64_steps", type=int, default=1)
    ap.add_argument("--L", type=int, default=None)
    ap.add_argument("--ref-L", dest="ref_L", type=int, default=4, help="helmholtz CPU sample level")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--breakdown", action="store_true")
    ap.add_argument("--workload", default="poisson", choices=sorted(WORKLOADS))
    ap.add_argument("--oracle", action="store_true", help="c4: also run the FP64 CPU oracle (minutes)")
    ap.add_argument("--no-autotune", dest="no_autotune", action="store_true",
                    help="skip the GEMM autotuner (built-in kernel choices)")
    ap.add_argument("--train-fronts", dest="train_fronts", type=int, default=6, help="c5: fronts to train on")
    ap.add_argument("--threshold", type=float, default=0.9, help="c5: proposal probability threshold")
    args = ap.parse_args()
    wl = WORKLOADS[args.workload]
    if args.L is None:
        args.L = wl["L"]
    if args.impl == "reference":
        return run_reference(args)
    if args.workload in ("c1", "c4", "c5"):
        return {"c1": run_c1, "c4": run_c4, "c5": run_c5}[args.workload](args)

    import torch

    import jaxhps_gb300 as hps
    from jaxhps_gb300 import _native as nat
    from jaxhps_gb300 import _phases as phases

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    L, p, q, ns = args.L, wl["p"], wl["q"], wl["nsrc"]
    if args.workload == "helmholtz":
        dom, coeffs, f, g = make_inputs_helmholtz(L, p, q, wl["k"], dev)
    else:
        dom, coeffs, f, g = make_inputs(L, p, q, ns, dev)
    arrays = {k: v for k, v in coeffs.items() if isinstance(v, torch.Tensor)}
    flags = {k: v for k, v in coeffs.items() if not isinstance(v, torch.Tensor)}
    n_leaves = dom.n_leaves
    pde = hps.PDEProblem(dom, source=f, **coeffs)

    def step():
        pde.reset()
        hps.build_solver(pde, precision=args.precision)
        return hps.solve(pde, g, host_device=None)

    # tile shapes and kernels of the products from the project's autotuner
    # (untimed): every variant timed on every product shape of one step
    tuning = None
    if not args.no_autotune:
        from jaxhps_gb300 import autotune

        rep = autotune.tune(step, reps=3)
        names = {}
        for sh in rep["shapes"]:
            names[sh["variant_name"]] = names.get(sh["variant_name"], 0) + 1
        tuning = {"shapes": len(rep["shapes"]), "seconds": rep["seconds"], "variants": names,
                  "builtin_ms_sum": rep["builtin_total_ms"], "tuned_ms_sum": rep["tuned_total_ms"]}
        pde.reset()
        nat.release_workspace()
        torch.cuda.empty_cache()

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    clocks = ClockSampler()
    clocks.start()
    launches0 = nat.launch_count()
    nat.profile_begin(nat.KC_GEMM, nat.KC_INVERSE, nat.KC_MOVE, nat.KC_RESIDUAL, nat.KC_GEMM_TMA,
                      nat.KC_RESIDUAL_DF, nat.KC_INVERSE_TC)
    barrier()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.nvtx.range_push("timed")   # lets a profiler select the timed steps
    e0.record()
    for _ in range(args.steps):
        u = step()
    e1.record()
    torch.cuda.nvtx.range_pop()
    torch.cuda.synchronize()
    barrier()
    ms = e0.elapsed_time(e1)
    classes = nat.profile_end()
    launches = nat.launch_count() - launches0
    clk = clocks.stop()
    if world > 1:
        ms = max_over_ranks(ms, dev)
    ms_per_step = ms / args.steps
    value = world * n_leaves / (ms_per_step / 1e3)
    iters = len(pde._state.history) if getattr(pde, "_state", None) is not None else None
    history = [float(h) for h in pde._state.history] if iters else None
    pde.reset()                      # the comparison run below needs the memory
    nat.release_workspace()
    torch.cuda.empty_cache()

    # e2e through the public API from pinned host memory
    e2e = None
    if not args.no_e2e:
        hf = f.cpu().pin_memory()
        hg = g.cpu().pin_memory()
        hco = {k: v.cpu().pin_memory() for k, v in arrays.items()}
        h2d = (hf.numel() * hf.element_size() + hg.numel() * hg.element_size() +
               sum(v.numel() * v.element_size() for v in hco.values()))
        d2h = n_leaves * p * p * ns * u.element_size()
        pde_h = hps.PDEProblem(dom, source=hf, **hco, **flags)

        # the caller's page-locked result buffer, reused every call
        hu = torch.empty(tuple(u.shape), dtype=u.dtype).pin_memory()

        def estep():
            pde_h.reset()
            hps.build_solver(pde_h, precision=args.precision)
            return hps.solve(pde_h, hg, out=hu)

        # warm-up calls (as many as the device-resident warm-up, at least
        # three); the first copies into a fresh page-locked block run at a
        # fraction of the link speed
        for _ in range(max(3, args.warmup)):
            uh = estep()
        torch.cuda.synchronize()
        n_e2e = max(5, args.steps)
        t0 = time.perf_counter()
        for _ in range(n_e2e):
            uh = estep()
        torch.cuda.synchronize()
        te = (time.perf_counter() - t0) / n_e2e
        if world > 1:
            barrier()
            te = max_over_ranks(te, dev)
        e2e = {"value": world * n_leaves / te, "unit": "leaves/s", "h2d_bytes_per_step": int(h2d),
               "d2h_bytes_per_step": int(d2h), "ms_per_step": te * 1e3}
        # where an end-to-end call spends its time: CUDA events at the phase
        # boundaries of build_solver / solve, a separate pass after the timed one
        phase_ms: dict = {}
        n_ph = 3
        phases.enable()
        for _ in range(n_ph):
            phases.mark("start")
            estep()
            for k, v in phases.collect().items():
                phase_ms[k] = phase_ms.get(k, 0.0) + v / n_ph
        phases.disable()
        e2e["phases_ms"] = phase_ms
        del pde_h, uh, hu
        nat.release_workspace()
        torch.cuda.empty_cache()

    # the plain FP64 GPU path on the same problem: its rate, and the error of
    # this run's solution against it
    err, fp64, u64_host = None, None, None
    u_host = u.cpu().numpy()
    if args.precision != "float64":
        pde64 = hps.PDEProblem(dom, source=f, **coeffs)
        torch.cuda.synchronize()
        b0, b1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        b0.record()
        hps.build_solver(pde64, precision="float64")
        u64 = hps.solve(pde64, g, host_device=None)
        b1.record()
        torch.cuda.synchronize()
        err = float(((u - u64).abs().max() / u64.abs().max()).item())
        u64_host = u64.cpu().numpy()
        if args.fp64_steps <= 0:
            ms64 = b0.elapsed_time(b1)
            fp64 = {"value": n_leaves / (ms64 / 1e3), "unit": "leaves/s", "ms_per_step": ms64,
                    "speedup_of_this_path": ms64 / ms_per_step, "note": "one run, the first of this path"}
        else:
            torch.cuda.synchronize()
            a0, a1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a0.record()
            for _ in range(args.fp64_steps):
                pde64.reset()
                hps.build_solver(pde64, precision="float64")
                u64 = hps.solve(pde64, g, host_device=None)
            a1.record()
            torch.cuda.synchronize()
            ms64 = a0.elapsed_time(a1) / args.fp64_steps
            fp64 = {"value": n_leaves / (ms64 / 1e3), "unit": "leaves/s", "ms_per_step": ms64,
                    "speedup_of_this_path": ms64 / ms_per_step}
        del pde64, u64
        nat.release_workspace()
        torch.cuda.empty_cache()
    del u
    torch.cuda.empty_cache()

    peaks = {}
    pk = ROOT / "MEASURED_PEAKS.json"
    if pk.exists():
        peaks = json.loads(pk.read_text())
    breakdown = {CLASS_NAMES[c]: {"ms_per_step": v[0] / args.steps, "share": v[0] / ms, "launches_per_step":
                                  v[1] / args.steps} for c, v in classes.items()}
    mhz = (clk or {}).get("sm_mhz") or 2070.0
    n_i = p * p - 4 * (p - 1)
    # algorithmic bytes of one FP64 residual launch: read u_int, g, f, coefficients; write r (pair), flux
    res_bytes = n_leaves * ns * (n_i * 8 + 4 * q * 8 + p * p * 8 + n_i * 8 + 4 * q * 8) + 3 * n_leaves * p * p * 8
    rooflines = {CLASS_NAMES[c]: class_roofline(nat, c, v, ms, peaks, mhz, res_bytes, args.workload, L)
                 for c, v in classes.items()}
    dom_cls = max(classes, key=lambda c: classes[c][0])
    roofline = dict(rooflines[CLASS_NAMES[dom_cls]])

    # the FP64 CPU oracle on the same inputs at the same size: the accuracy
    # reference and, timed, the CPU baseline
    cpu, acc = None, {}
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        if args.workload == "helmholtz":
            v, dt, n, what = _cpu_sample_helmholtz(args)
            cpu = {"value": v, "unit": "leaves/s", "cores": cpu_threads(), "kind": "port",
                   "sample": f"{what}, {dt:.1f} s"}
        else:
            c_h = coeffs["I_coefficients"].cpu().numpy()
            u_o, dt = oracle_poisson(c_h, f.cpu().numpy(), g.cpu().numpy(), L, p, q)
            speedup = oracle_thread_speedup(L=min(5, L), p=p, q=q, nsrc=ns)
            cpu = {"value": n_leaves / dt, "unit": "leaves/s", "cores": cpu_threads(), "kind": "port",
                   "thread_speedup": speedup,
                   "sample": (f"the full workload (L={L}, {n_leaves} leaves, {ns} RHS) once, {dt:.1f} s: "
                              f"level-batched FP64 NumPy oracle on every host thread (an L={min(5, L)} instance runs "
                              f"{speedup:.1f}x faster on all threads than on one)")}

            def errs(a, b):
                return {"rel_l2": float(np.linalg.norm((a - b).ravel()) / np.linalg.norm(b.ravel())),
                        "rel_linf": float(np.abs(a - b).max() / np.abs(b).max())}

            e = errs(u_host, u_o)
            acc = {"rel_l2_vs_oracle": e["rel_l2"], "rel_linf_vs_oracle": e["rel_linf"]}
            if u64_host is not None:
                acc["fp64_path_vs_oracle"] = errs(u64_host, u_o)
            del u_o

    if args.workload == "helmholtz":
        dtype = {"float64": "c128", "float32": "c64", "mixed": "c64+c128-refinement"}[args.precision]
    else:
        dtype = {"float64": "f64", "float32": "f32", "mixed": "f32+f64-refinement"}[args.precision]
    line = {
        "metric": "build+solve leaves/s", "value": value, "unit": "leaves/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": dtype, "data": "synthetic",
        "config": {"workload": wl["name"], "L": L, "n_leaves": n_leaves, "p": p, "q": q, "nsrc": ns,
                   "precision": args.precision, "parallelism": "replicas" if world > 1 else "single-gpu",
                   "l2": "inputs larger than L2 (operator set is several GB)"},
        "rel_err_vs_fp64": err, **acc, "refinement_iterations": iters,
        "refinement_history": history, "fp64_path": fp64,
        "e2e": e2e, "gpu_launches": launches, "roofline": roofline, "kernel_classes": breakdown,
        "kernel_rooflines": rooflines,
        "cpu_baseline": cpu, "clocks": clk, "autotune": tuning,
    }
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
