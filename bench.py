"""Design iterations per second of pyMOTO's 3D compliance path on GB300.

Workload (one "step" = one design iteration): 3D cantilever, hex8 128x64x64 (1,635,075 dofs), E0=1,
nu=0.3, SIMP p=3 (xmin=1e-9), FilterConv r=2.5, left face clamped, unit -y point load at node
(128,32,32); FilterConv -> SIMP -> K(x) -> multigrid-PCG to relative residual 1e-6 (warm-started from
the previous solution) -> compliance -> adjoint (LDA projection) -> sensitivity -> filter transpose ->
OC update (move 0.2), all on the device.  Initial density: seeded U(1e-3, 1).

Arms: "plain_fp64" (FP64 CG with an FP64 geometric-multigrid preconditioner, pyMOTO's algorithm), "mixed"
(FP64 flexible CG around FP32 PCG iterations with an FP32 multigrid preconditioner) and the headline
"mixed_learned" (the mixed arm with the learned warm start, as the metric is defined).  `value` is the
headline arm (the mixed arm when the learned one is not run).  `--impl reference` times the CPU restatement of
pyMOTO's own path (oracle) on the host cores.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
"""
import os

# the CPU baseline and the reference arm use every host core (numpy/scipy BLAS and OpenMP pools are sized at
# import, so this precedes the numpy import)
for _v in ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS", "MKL_NUM_THREADS"):
    os.environ.setdefault(_v, str(os.cpu_count() or 1))

import argparse  # noqa: E402
import json  # noqa: E402
import statistics  # noqa: E402
import subprocess  # noqa: E402
import sys  # noqa: E402
import threading  # noqa: E402
import time  # noqa: E402

import numpy as np  # noqa: E402

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "design iters/s, hex8 128×64×64 @1e-6 residual: learned+mixed vs plain FP64 PCG"
SHAPE = (128, 64, 64)
RADIUS, PENAL, XMIN, TOL, MOVE, OMEGA, SWEEPS = 2.5, 3.0, 1e-9, 1e-6, 0.2, 0.6, 2
GPU_LEVELS = 5          # 128x64x64 -> 8x4x4 coarsest (675 dofs, dense FP64 Cholesky + explicit inverse)
REF_LEVELS = 4          # the reference example's hierarchy: coarsest 16x8x8 (SuperLU)
L2_FLUSH_BYTES = 256 << 20
# DRAM bytes (read + write) per launch of the roofline kernel at the bench workload, from the ncu capture
# summarised in profiles/ebe_apply_tc_residual_hex8_128x64x64.md
NCU_TRAFFIC_PER_LAUNCH = {"ebe_apply_tc_residual_f32": 15.756e6, "ebe_apply_fma_residual_f32": 15.772e6}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--shape", default=None, help="override the grid, e.g. 64x32x32")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--timed-only", action="store_true",
                    help="stop after the timed design iterations (no parity, e2e or kernel timing): for launch lists")
    ap.add_argument("--profile-breakdown", action="store_true", help="print a per-kernel time table")
    ap.add_argument("--inner-iters", type=int, default=6, help="FP32 PCG iterations per FCG preconditioning")
    ap.add_argument("--inner-tol", type=float, default=0.1)
    ap.add_argument("--fcg-m", type=int, default=1)
    ap.add_argument("--levels", type=int, default=GPU_LEVELS)
    ap.add_argument("--sweeps", type=int, default=SWEEPS)
    ap.add_argument("--coarse-sweeps", type=int, default=None)
    ap.add_argument("--case", default=None, choices=["operator", "mma", "mma_run", "poisson"],
                    help="instead of the bench: time the level-0 operator kernels alone (a small case for ncu), "
                         "the device MMA update of the 96x48x48 design against the numpy MMA, the 96x48x48 "
                         "MMA workload (mma_run), or thermal design evaluations on the one-component operator "
                         "(poisson)")
    ap.add_argument("--mma-iters", type=int, default=100, help="MMA iterations of --case mma_run")
    ap.add_argument("--pretrain", type=int, default=256,
                    help="smoothed-noise fields the learned warm start sees before --case mma_run")
    ap.add_argument("--arms", default="plain_fp64,plain_fp64_cheb,mixed,mixed_learned",
                    help="plain_fp64 (the reference's method), plain_fp64_cheb (its smoother ablation: FP64 with "
                         "the mixed arm's Chebyshev smoother), mixed, mixed_learned (headline: with the learned "
                         "warm start), ablation mixed_jacobi")
    ap.add_argument("--cpu-steps", type=int, default=5, help="warm design iterations of the CPU baseline (median)")
    return ap.parse_args()


def dist_info():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


# ------------------------------------------------------------------------------------------ replicas
# The path does not shard across GPUs here (one GPU per box): N ranks run N independent design loops with
# their own seeds; the only collectives are a barrier around the timed region and the maximum of the timed
# totals over the ranks.
def replica_seed(rank):
    return 1234 + rank


def max_over_ranks(v, world, device):
    """The largest value of v over the ranks (v itself with one rank)."""
    if world <= 1:
        return v
    import torch
    t = torch.tensor([v], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def aggregate_rate(world, steps, slowest_total_s):
    """Whole-job design iterations per second: every rank did `steps`, the job took the slowest rank's time."""
    return world * steps / slowest_total_s


# ------------------------------------------------------------------------------------------ problem
def cantilever(shape):
    nx, ny, nz = shape
    nnx, nny = nx + 1, ny + 1
    left = np.array([(k * nny + j) * nnx for k in range(nz + 1) for j in range(nny)], dtype=np.int64)
    bc = (left[:, None] * 3 + np.arange(3)).ravel()
    f = np.zeros((nx + 1) * (ny + 1) * (nz + 1) * 3)
    tip = ((nz // 2) * nny + ny // 2) * nnx + nx
    f[3 * tip + 1] = -1.0
    return bc, f


class DesignRun:
    """The network of the workload on the device, for one solver arm."""

    opts = {"inner_iters": 6, "inner_tol": 0.1, "m": 1, "levels": GPU_LEVELS, "sweeps": SWEEPS, "coarse_sweeps": None,
            "smoother": "chebyshev", "cheb_degree": 1, "cheb_coarse_degree": [2, 3, 4], "cheb_ratio": 15.0,
            "learned_train_steps": 1, "learned_stride": 4, "learned_lr": 2e-3, "learned_net": True,
            "learned_history": 0, "learned_train_every": 4, "learned_gate": 0.02, "learned_gate_skip": 3,
            "learned_cc": False,
            "coarse_lag": True}

    def __init__(self, arm, shape, seed, torch, pg):
        o = DesignRun.opts
        self.arm = arm
        d = pg.VoxelDomain(*shape)
        bc, f = cantilever(shape)
        self.nel = d.nel
        rng = np.random.default_rng(seed)
        x0 = rng.uniform(1e-3, 1.0, d.nel)
        self.f = torch.from_numpy(f).cuda()
        self.sx = pg.Signal("x", torch.from_numpy(x0).cuda())
        # arms: plain_fp64 = the reference's method (FP64 CG + FP64 GMG, damped Jacobi w=0.6, 2 sweeps) on the
        # GPU; mixed = FP64 FCG + FP32 GMG with the Chebyshev smoother; the *_cheb / *_jacobi variants are
        # the ablations (smoother swapped)
        mixed = arm.startswith("mixed")
        cheb = (mixed and arm != "mixed_jacobi" and o["smoother"] == "chebyshev") or arm == "plain_fp64_cheb"
        self.smoother = "chebyshev" if cheb else "jacobi"
        with pg.Network() as fn:
            xf = pg.FilterConv(d, radius=RADIUS)(self.sx)
            xs = pg.SIMP(xmin=XMIN, penal=PENAL)(xf)
            K = pg.AssembleStiffness(d, bc=bc, sensitivity_precision="mixed" if mixed else "fp64")(xs)
            if cheb:
                mgs = pg.GeometricMultigrid.hierarchy(d, levels=o["levels"], smooth_steps=o["cheb_degree"],
                                                      precision="fp32" if mixed else None,
                                                      coarse_smooth_steps=o["cheb_coarse_degree"],
                                                      smoother="chebyshev", cheb_ratio=o["cheb_ratio"],
                                                      coarse_lag=o["coarse_lag"] and mixed)
            else:
                mgs = pg.GeometricMultigrid.hierarchy(d, levels=o["levels"], smoother_w=OMEGA,
                                                      smooth_steps=o["sweeps"], precision="fp32" if mixed else None,
                                                      coarse_smooth_steps=o["coarse_sweeps"])
            if mixed:
                self.warm_start = None
                if arm == "mixed_learned":
                    from pymoto_gb300.learned import LearnedWarmStart
                    self.warm_start = LearnedWarmStart(shape, stride=o["learned_stride"], capacity=8,
                                                       train_steps=o["learned_train_steps"], lr=o["learned_lr"],
                                                       seed=seed, use_net=o["learned_net"],
                                                       history=o["learned_history"],
                                                       train_every=o["learned_train_every"],
                                                       gate=o["learned_gate"], gate_skip=o["learned_gate_skip"],
                                                       coarse_correction=o["learned_cc"])
                # stops on the recursive FP64 residual like the plain arm's CG (the true residual of every timed
                # solve is recomputed outside the timed region and reported)
                self.solver = pg.MixedPrecisionCG(preconditioner=mgs[0], tol=TOL, m=o["m"], inner_iters=o["inner_iters"],
                                                  inner_tol=o["inner_tol"], warm_start=self.warm_start,
                                                  verify_residual=False)
            else:
                self.solver = pg.CG(preconditioner=mgs[0], tol=TOL)
            self.u = pg.LinSolve(hermitian=True, symmetric=True, solver=self.solver)(K, self.f)
            self.c = pg.EinSum("i,i->")(self.u, self.f)
        self.fn = fn
        self.K = K
        self.oc = pg.OC(self.sx, self.c, fn, move=MOVE, verbosity=0)
        self.iters = []

    def step(self):
        self.oc.step()
        self.iters.append(self.solver.iterations)


def design_solution(arm, shape, x, tol, torch, pg):
    """c, u, dc/dx (host arrays) of one design x on the GPU: arm 'fp64' (CG + FP64 GMG, damped Jacobi 0.6, 2 sweeps,
    the plain arm's solver) or 'mixed' (the mixed arm's solver); the true FP64 relative residual."""
    o = DesignRun.opts
    d = pg.VoxelDomain(*shape)
    bc, f = cantilever(shape)
    fd = torch.from_numpy(f).cuda()
    sx = pg.Signal("x", torch.from_numpy(np.ascontiguousarray(x)).cuda())
    mixed = arm == "mixed"
    with pg.Network() as fn:
        xf = pg.FilterConv(d, radius=RADIUS)(sx)
        xs = pg.SIMP(xmin=XMIN, penal=PENAL)(xf)
        K = pg.AssembleStiffness(d, bc=bc, sensitivity_precision="mixed" if mixed else "fp64")(xs)
        if mixed:
            mgs = pg.GeometricMultigrid.hierarchy(d, levels=o["levels"], smooth_steps=o["cheb_degree"], precision="fp32",
                                                  coarse_smooth_steps=o["cheb_coarse_degree"], smoother="chebyshev",
                                                  cheb_ratio=o["cheb_ratio"])
            solver = pg.MixedPrecisionCG(preconditioner=mgs[0], tol=tol, m=o["m"], inner_iters=o["inner_iters"],
                                         inner_tol=o["inner_tol"])
        else:
            mgs = pg.GeometricMultigrid.hierarchy(d, levels=o["levels"], smoother_w=OMEGA, smooth_steps=o["sweeps"])
            solver = pg.CG(preconditioner=mgs[0], tol=tol, maxit=10000)
        lin = pg.LinSolve(hermitian=True, symmetric=True, solver=solver)
        u = lin(K, fd)
        c = pg.EinSum("i,i->")(u, fd)
    fn.reset()
    c.sensitivity = 1.0
    fn.sensitivity()
    res = pg.LinearSolver.residual(lin.A, lin._u_dev, fd)
    return {"c": float(c.state), "u": u.state.cpu().numpy(), "dc": sx.sensitivity.cpu().numpy(), "residual": res,
            "tol": tol}


def parity_errors(sol, ref):
    """Relative errors of a GPU solution against the oracle's: |c - c*| / |c*|, ||u - u*|| / ||u*||,
    max |dc - dc*| / max |dc*|."""
    return {"c": abs(sol["c"] - ref["c"]) / abs(ref["c"]),
            "u": float(np.linalg.norm(sol["u"] - ref["u"]) / np.linalg.norm(ref["u"])),
            "dc": float(np.abs(sol["dc"] - ref["dc"]).max() / np.abs(ref["dc"]).max()),
            "gpu_true_rel_residual": sol["residual"], "gpu_tol": sol["tol"]}


class ClockSampler:
    """nvidia-smi samples (SM clock, throttle reasons) while the timed region runs."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
            # the sampler is live before the timed region starts (nvidia-smi takes a moment to print its first
            # line); the wait is bounded, a sampler that never prints leaves "samples": 0
            t0 = time.time()
            while not self.lines and self.proc.poll() is None and time.time() - t0 < 10.0:
                time.sleep(0.02)
            self.lines.clear()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            p = [v.strip() for v in ln.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                smax = float(p[2])
            except ValueError:
                continue
            for nm, v in zip(names, p[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def time_arm(run, steps, warmup, torch, flush, probe_targets=None, pg=None):
    """Warm up, then time `steps` design iterations with CUDA events (L2 flushed before each step)."""
    for _ in range(warmup):
        run.step()
    torch.cuda.synchronize()
    run.iters.clear()
    durs = []
    probe = pg._lib.Probe(targets=probe_targets) if pg is not None else None
    if probe is not None:
        probe.__enter__()
    try:
        for _ in range(steps):
            flush.zero_()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
            run.step()
            e1.record()
            torch.cuda.synchronize()
            durs.append(e0.elapsed_time(e1))
    finally:
        if probe is not None:
            probe.__exit__()
    return durs, probe


def headline_arm(results):
    """The arm `value` reports: the learned + mixed-precision arm of the metric, else the mixed one."""
    return "mixed_learned" if "mixed_learned" in results else "mixed"


def kernel_rooflines(run, flush, torch, reps=20):
    """Live CUDA-event times of the level-0 operator kernels on the headline arm's final operators, one launch at
    a time on the current stream with the L2 flushed (256 MB write) before each launch:
      * the FP32 matrix-free operator in residual mode, the most launched kernel of a design iteration (one
        matvec, one residual and one Chebyshev step per inner iteration), in both implementations: FP32 FMAs on
        the CUDA cores ("fma") and 3xTF32 tcgen05.mma products ("tcgen05");
      * the FP64 node-stencil product (the outer FCG operator), whose bound is the FP64 pipe.
    Returns per kernel: seconds per launch, algorithmic bytes and flops per launch."""
    import pymoto_gb300 as pg
    from pymoto_gb300._lib import MATVEC, RESIDUAL
    sol = run.solver
    A32, A64 = sol.A32, sol.A64
    g = A64.grid
    nel, nn, ndof = g.nel, g.nnodes, g.ndof
    u32 = torch.randn(ndof, device="cuda")
    b32, y32 = torch.randn_like(u32), torch.empty_like(u32)
    u64 = torch.randn(ndof, dtype=torch.float64, device="cuda")
    y64 = torch.empty_like(u64)

    def timed(fn):
        fn()
        torch.cuda.synchronize()
        tot = 0.0
        for _ in range(reps):
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            fn()
            e1.record()
            torch.cuda.synchronize()
            tot += e0.elapsed_time(e1)
        return tot / reps * 1e-3

    out = {"selected": pg.operator_kernel()}
    for kind in ("fma", "tcgen05"):
        prev = pg.set_operator_kernel(kind)
        t = timed(lambda: A32.apply(RESIDUAL, u32, b32, out=y32))
        pg.set_operator_kernel(prev)
        # u, b read and y written once (FP32), element scaling (FP32) and the node constraint mask (bytes);
        # 24 x 24 FMAs per element (the tensor-core form runs three TF32 products of that size)
        out[f"ebe_apply_{kind}_residual_f32"] = {"s": t, "bytes": 3 * 4 * ndof + 4 * nel + nn,
                                                 "flops": 2 * 24 * 24 * nel}
    t = timed(lambda: A64.apply(MATVEC, u64, out=y64))
    # 27 blocks of 3 x 3 per row of 3 dofs: 81 FP64 FMA per dof; stored stencils (14 blocks) + u + y once
    out["stencil_apply_f64_matvec"] = {"s": t, "bytes": 8 * (126 * nn + 2 * ndof), "flops": 2 * 81 * ndof}
    return out


def measure_gb300(args, rank, world, local_rank):
    import torch
    import pymoto_gb300 as pg

    torch.cuda.set_device(local_rank)
    shape = SHAPE if args.shape is None else tuple(int(v) for v in args.shape.split("x"))
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    peaks = {}
    pth = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(pth):
        with open(pth) as fh:
            peaks = json.load(fh)
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    peak_src = "measured" if "hbm_gbs" in peaks else "fallback"

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    def slowest(v):
        return max_over_ranks(v, world, "cuda")

    DesignRun.opts.update({"inner_iters": args.inner_iters, "inner_tol": args.inner_tol, "m": args.fcg_m,
                           "levels": args.levels, "sweeps": args.sweeps, "coarse_sweeps": args.coarse_sweeps})
    results = {}
    for arm in args.arms.split(","):
        run = DesignRun(arm, shape, seed=replica_seed(rank), torch=torch, pg=pg)
        targets = set()          # count launches only: no events inside the timed region
        barrier()
        torch.cuda.synchronize()
        with ClockSampler(local_rank) as clk:
            durs, probe = time_arm(run, args.steps, args.warmup, torch, flush, targets, pg)
        barrier()
        total = slowest(sum(durs))
        results[arm] = {"durs": durs, "total_ms": total, "iters": list(run.iters), "probe": probe,
                        "clocks": clk.summary(), "run": run}
        # true FP64 residual of the last solve
        A = run.K.state if hasattr(run.K, "state") else None
        lin = run.fn.mods[3]
        res = pg.LinearSolver.residual(lin.A, lin._u_dev, run.f)
        results[arm]["true_residual"] = res
        results[arm]["compliance"] = float(run.c.state)

    if args.timed_only:           # profiling runs: the timed design iterations and nothing after them
        if rank == 0:
            print(json.dumps({"timed_only": True, "arms": {a: {"ms_per_step": r["total_ms"] / args.steps,
                                                               "solver_iterations": r["iters"]}
                                                           for a, r in results.items()}}))
        return None
    # same-design parity: solve the plain arm's final design with both solvers
    run_p = results[next(iter(results))]["run"]
    lin_p = run_p.fn.mods[3]
    A = lin_p.A
    b = run_p.f.clone()
    mask = torch.empty_like(b)
    pg._lib.call("pmg_mask_bc", 0, 3, A.grid.nnodes, A.bcmask, 0, b, mask, pg._lib.stream())
    o = DesignRun.opts
    mgs = pg.GeometricMultigrid.hierarchy(pg.VoxelDomain(*shape), levels=args.levels, smooth_steps=o["cheb_degree"],
                                          precision="fp32", coarse_smooth_steps=o["cheb_coarse_degree"],
                                          smoother="chebyshev", cheb_ratio=o["cheb_ratio"])
    ms = pg.MixedPrecisionCG(preconditioner=mgs[0], tol=TOL, m=args.fcg_m, inner_iters=args.inner_iters,
                             inner_tol=args.inner_tol)
    ms.update(A)
    u_m = ms.solve(mask)
    mgs64 = pg.GeometricMultigrid.hierarchy(pg.VoxelDomain(*shape), levels=args.levels, smoother_w=OMEGA,
                                            smooth_steps=SWEEPS)
    tight = pg.CG(preconditioner=mgs64[0], tol=1e-11)
    tight.update(A)
    u_t = tight.solve(mask)
    c_m = float(torch.dot(mask, u_m).item())
    c_t = float(torch.dot(mask, u_t).item())

    # end-to-end through the public API with host buffers, on the same designs as the timed region: a second run
    # of the headline arm from the same seed replays the warm-up designs (every kernel and reduction is
    # deterministic), then each timed step copies the step's design from pinned host memory to the device, runs
    # the design iteration and copies the compliance and the new design back
    H = headline_arm(results)
    run = DesignRun(H, shape, seed=replica_seed(rank), torch=torch, pg=pg)
    for _ in range(args.warmup):
        run.step()
    nel = run.nel
    x_host = torch.empty(nel, dtype=torch.float64).pin_memory()
    x_host.copy_(run.sx.state.cpu())
    c_host = torch.empty(1, dtype=torch.float64).pin_memory()
    run.iters.clear()
    barrier()
    torch.cuda.synchronize()
    e2e_durs = []
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        run.sx.state = x_host.to("cuda", non_blocking=True)          # H2D of the step's design
        run.step()
        c_host.copy_(run.c.state.reshape(1) if isinstance(run.c.state, torch.Tensor)
                     else torch.tensor([float(run.c.state)]), non_blocking=True)   # D2H of the compliance
        x_host.copy_(run.sx.state, non_blocking=True)                  # D2H of the new design
        torch.cuda.synchronize()
        e2e_durs.append(time.perf_counter() - t0)
    e2e_total = slowest(sum(e2e_durs))
    e2e_same = run.iters == results[H]["iters"]

    # the first design of the timed runs (same seed) solved by both GPU solvers, for the oracle comparison of the
    # CPU-baseline leg
    design1 = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        x1 = np.random.default_rng(replica_seed(0)).uniform(1e-3, 1.0, int(np.prod(shape)))
        design1 = {"x": x1, "fp64": design_solution("fp64", shape, x1, 1e-10, torch, pg),
                   "mixed": design_solution("mixed", shape, x1, TOL, torch, pg)}
    kernels = kernel_rooflines(results[headline_arm(results)]["run"], flush, torch) if rank == 0 else None
    out = {"results": results, "shape": shape, "hbm_peak": hbm_peak, "peak_src": peak_src, "c_mixed": c_m,
           "c_tight": c_t, "e2e_total_s": e2e_total, "e2e_same_designs": e2e_same, "e2e_iters": list(run.iters), "nel": nel, "res_mixed_same_design": ms.last_residual,
           "kernels": kernels, "peaks": peaks, "design1": design1}
    if args.profile_breakdown and rank == 0:
        run = DesignRun("mixed", shape, seed=99, torch=torch, pg=pg)
        for _ in range(2):
            run.step()
        torch.cuda.synchronize()
        with pg._lib.Probe(targets=None) as pr:
            for _ in range(3):
                run.step()
        torch.cuda.synchronize()
        out["breakdown"] = pr.summary()
    return out


def cpu_reference_sample(shape, warm_steps=1, warmup=1, seed=1234):
    """Time `warm_steps` design iterations of the CPU restatement after `warmup` untimed ones (the first is the
    cold solve), from the GPU arms' initial design (same seed)."""
    import oracle
    L = oracle.ReferenceDesignLoop(shape, radius=RADIUS, levels=REF_LEVELS, w=OMEGA, smooth_steps=SWEEPS, tol=TOL,
                                   move=MOVE, seed=seed)
    for _ in range(max(1, warmup)):
        L.step()                   # cold solve and warm-up, untimed
    times = []
    for _ in range(warm_steps):
        t0 = time.perf_counter()
        L.step()
        times.append(time.perf_counter() - t0)
    return times, L


def operator_case(args):
    """Operator products of the workload alone: the FP32 level-0 operator in residual mode (CUDA-core and
    tensor-core implementations), FP64 stencil product, FP32 level-1 stencil residual, and the one-component
    (Poisson) operator's FP64 product, FP32 residual and FP64 Galerkin product on the same grid; 3 launches each
    after 2 warm-up launches, CUDA-event times printed as JSON (a small case for ncu)."""
    import torch
    import pymoto_gb300 as pg
    from pymoto_gb300._lib import F32, RESIDUAL, MATVEC
    shape = SHAPE if args.shape is None else tuple(int(v) for v in args.shape.split("x"))
    d = pg.VoxelDomain(*shape)
    bc, f = cantilever(shape)
    x = torch.from_numpy(np.random.default_rng(0).uniform(1e-3, 1.0, d.nel) ** 3).cuda()
    K = pg.AssembleStiffness(d, bc=bc)(x)
    K32 = K.astype(F32)
    u = torch.randn(K.grid.ndof, dtype=torch.float64, device="cuda")
    u32, b32 = u.float(), torch.randn_like(u.float())
    A1 = K32.galerkin()            # level 1 (FP32 Galerkin stencils, half-symmetric)
    u1 = torch.randn(A1.grid.ndof, device="cuda")
    b1 = torch.randn_like(u1)
    # the one-component (Poisson) operator on the same grid and element scaling
    from pymoto_gb300.operators import ScalarOperator, element_poisson
    nn = K.grid.nnodes
    P = ScalarOperator.assemble(K.grid, x, element_poisson(d, 1.0), torch.zeros(nn, dtype=torch.uint8, device="cuda"),
                                1.0)
    P32 = P.astype(F32)
    Pc = P.galerkin()
    v64, v32, c32 = torch.randn(nn, dtype=torch.float64, device="cuda"), torch.randn(nn, device="cuda"), \
        torch.randn(nn, device="cuda")
    out = {}

    def with_kernel(kind, fn):
        def run():
            prev = pg.set_operator_kernel(kind)
            fn()
            pg.set_operator_kernel(prev)
        return run

    for name, fn in [("ebe_apply_fma_f32_residual", with_kernel("fma", lambda: K32.apply(RESIDUAL, u32, b32))),
                     ("ebe_apply_tc_f32_residual", with_kernel("tcgen05", lambda: K32.apply(RESIDUAL, u32, b32))),
                     ("stencil_apply_f64_matvec", lambda: K.apply(MATVEC, u)),
                     ("stencil_apply_f32_level1_residual", lambda: A1.apply(RESIDUAL, u1, b1)),
                     ("scalar_apply_f64_matvec", lambda: P.apply(MATVEC, v64)),
                     ("scalar_apply_f32_residual", lambda: P32.apply(RESIDUAL, v32, c32)),
                     ("scalar_galerkin_f64", lambda: P.galerkin(out=Pc))]:
        for _ in range(2):
            fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(3):
            fn()
        e1.record()
        torch.cuda.synchronize()
        out[name + "_us"] = e0.elapsed_time(e1) / 3 * 1e3
    prev = pg.set_operator_kernel("fma")
    ya = K32.apply(RESIDUAL, u32, b32)
    pg.set_operator_kernel("tcgen05")
    yb = K32.apply(RESIDUAL, u32, b32)
    pg.set_operator_kernel(prev)
    out["fma_vs_tc_max_rel_diff"] = float((ya - yb).abs().max() / yb.abs().max())
    print(json.dumps({"case": "operator", "shape": list(shape), **out}))


def heat_sink(shape):
    """Thermal load case: the middle half of the x = 0 face held at zero temperature, a uniform heat load."""
    nx, ny, nz = shape
    jj = np.arange(ny // 4, 3 * ny // 4 + 1)
    kk = np.arange(nz // 4, 3 * nz // 4 + 1)
    J, K = np.meshgrid(jj, kk, indexing="ij")
    nodes = ((K * (ny + 1) + J) * (nx + 1)).ravel()
    nn = (nx + 1) * (ny + 1) * (nz + 1)
    return nodes, np.full(nn, 1.0 / nn)


def poisson_case(args):
    """Thermal compliance evaluations on the one-component operator (AssemblePoisson, pymoto/modules/assembly.py:
    523-560): per step, P(x) assembled from a new design, LinSolve with CG and a 5-level FP64 multigrid (pyMOTO's
    method: damped Jacobi w = 0.6, 2 sweeps) to 1e-8, c = f.u and dc/dx.  Also: the one-component kernels timed
    alone (CUDA events, L2 flushed before each launch) against the measured HBM bandwidth, parity of the solve with
    the oracle on the last evaluation's design, whose run on the host cores is the CPU baseline."""
    import torch
    import pymoto_gb300 as pg
    import oracle as O
    from pymoto_gb300._lib import F32, F64, MATVEC, RESIDUAL
    from pymoto_gb300.operators import ScalarOperator, element_poisson
    shape = SHAPE if args.shape is None else tuple(int(v) for v in args.shape.split("x"))
    peaks = {}
    pth = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(pth):
        with open(pth) as fh:
            peaks = json.load(fh)
    hbm = peaks.get("hbm_gbs", 6800.0)
    tol = 1e-8

    def network(shp, x0):
        d = pg.VoxelDomain(*shp)
        nodes, f = heat_sink(shp)
        mgs = pg.GeometricMultigrid.hierarchy(d, levels=GPU_LEVELS, smoother_w=OMEGA,
                                              smooth_steps=SWEEPS)
        solver = pg.CG(preconditioner=mgs[0], tol=tol, maxit=500)
        fd = torch.from_numpy(f).cuda()
        sx = pg.Signal("x", torch.from_numpy(x0).cuda())
        with pg.Network() as fn:
            sK = pg.AssemblePoisson(d, bc=nodes)(sx)
            su = pg.LinSolve(hermitian=True, symmetric=True, solver=solver)(sK, fd)
            sc = pg.EinSum("i,i->")(su, fd)
        return fn, sx, sK, su, sc, solver

    rng = np.random.default_rng(0)
    nel = shape[0] * shape[1] * shape[2]
    x0 = rng.uniform(1e-3, 1.0, nel)
    fn, sx, sK, su, sc, solver = network(shape, x0)

    def step(k):
        sx.state = torch.from_numpy(np.clip(x0 * (1.0 + 0.02 * k), 1e-3, 1.0)).cuda()
        fn.response()
        fn.reset()
        sc.sensitivity = 1.0
        fn.sensitivity()

    for k in range(args.warmup):
        step(k)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    its = []
    with ClockSampler(0) as clk:
        e0.record()
        for k in range(args.steps):
            step(args.warmup + k)
            its.append(solver.iterations)
        e1.record()
        torch.cuda.synchronize()
    per = e0.elapsed_time(e1) / 1e3 / args.steps

    # kernels alone
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device="cuda")
    K = sK.state
    K32 = K.astype(F32)
    nn = K.grid.nnodes

    def timed(fn_, reps=20):
        for _ in range(3):
            fn_()
        ts = []
        for _ in range(reps):
            flush.fill_(1)
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            fn_()
            b.record()
            torch.cuda.synchronize()
            ts.append(a.elapsed_time(b) / 1e3)
        return statistics.median(ts)

    u64 = torch.randn(nn, dtype=torch.float64, device="cuda")
    u32, b32 = u64.float(), torch.randn(nn, dtype=torch.float32, device="cuda")
    y64, y32 = torch.empty_like(u64), torch.empty_like(u32)
    Kc = K.galerkin()
    kern = {}
    for name, fn_, nbytes in [
            ("scalar_apply_f64_matvec", lambda: K.apply(MATVEC, u64, out=y64), (27 + 2) * 8 * nn),
            ("scalar_apply_f32_residual", lambda: K32.apply(RESIDUAL, u32, b32, out=y32), (27 + 3) * 4 * nn),
            ("scalar_galerkin_f64", lambda: K.galerkin(out=Kc), 27 * 8 * (nn + Kc.grid.nnodes)),
            ("scalar_stencil_f64", lambda: K.recompute(), 27 * 8 * nn + 8 * nel + nn)]:
        t = timed(fn_)
        kern[name] = {"us": t * 1e6, "algorithmic_bytes": nbytes, "gbs": nbytes / t / 1e9,
                      "frac_of_measured_hbm": nbytes / t / 1e9 / hbm}

    # parity of the last timed evaluation with the oracle (same design, same grid), whose run is the CPU baseline
    x_last = np.clip(x0 * (1.0 + 0.02 * (args.warmup + args.steps - 1)), 1e-3, 1.0)
    u_gpu, dx_gpu, c_gpu = su.state.cpu().numpy(), sx.sensitivity.cpu().numpy(), float(sc.state)
    del flush, Kc, K32
    og = O.Grid(*shape)
    nodes, f = heat_sink(shape)
    P0 = element_poisson(pg.VoxelDomain(*shape), 1.0)
    t0 = time.perf_counter()
    A = O.assemble(og, P0, x_last, bc=nodes, bcdiagval=float(P0.max()), ndof=1).tocsr()
    lv = O.build_hierarchy(og, A, REF_LEVELS, w=OMEGA, smooth_steps=SWEEPS, ndof=1)
    u_ref, cpu_its, _ = O.cg_solve(A, f, precond=lambda r: O.vcycle(lv[0], r), tol=tol)
    dx_ref = O.sensitivity_contract(og, P0, [-u_ref], [u_ref], bc=nodes, ndof=1)
    t_cpu = time.perf_counter() - t0
    line = {"case": "poisson", "metric": "thermal design evaluations/s (assembly + CG/GMG solve to 1e-8 + c + dc/dx)",
            "value": 1.0 / per, "unit": "evaluations/s", "ms_per_step": per * 1e3, "steps": args.steps,
            "warmup": args.warmup, "dtype": "f64", "data": "synthetic (seeded U(1e-3,1) conductivities)",
            "config": {"workload": f"heat sink, one-component hex8 {shape[0]}x{shape[1]}x{shape[2]} "
                                   f"({nn} dofs), CG + FP64 GMG {GPU_LEVELS} levels, w={OMEGA}, {SWEEPS} sweeps",
                       "l2": "kernels: L2 flushed before each launch"},
            "cg_iterations": its, "kernels": kern, "clocks": clk.summary(),
            "parity": {"u_max_rel_diff": float(np.abs(u_gpu - u_ref).max() / np.abs(u_ref).max()),
                       "dx_max_rel_diff": float(np.abs(dx_gpu - dx_ref).max() / np.abs(dx_ref).max()),
                       "compliance_rel_diff": float(abs(c_gpu - f @ u_ref) / abs(f @ u_ref)),
                       "oracle_relative_residual_of_gpu_u": float(O.relative_residual(A, u_gpu, f))},
            "cpu_baseline": {"value": 1.0 / t_cpu, "unit": "evaluations/s", "cores": os.cpu_count() or 1,
                             "kind": "port", "sample": f"the last timed evaluation's design through the oracle "
                                                       f"(scipy assembly, SpGEMM Galerkin, {REF_LEVELS}-level GMG, "
                                                       f"SuperLU coarsest, CG {cpu_its} iterations, sensitivity) "
                                                       f"on the same grid: {t_cpu:.2f} s"}}
    print(json.dumps(line))


def mma_case(args):
    """The MMA update of a 96x48x48 design (221,184 variables, one volume constraint) on the device, fast and exact
    variants: 2 warm-up and 5 timed updates chained on their own output (CUDA events around each), then the numpy
    MMA of the oracle on the host cores for the first update with the same inputs, and the largest difference of
    the designs.  Synthetic compliance-like inputs: x ~ U(0.2, 0.8), objective 10 with dc/dx ~ -U(0, 20)/n,
    volume constraint mean(x) - 0.45 with gradient 1/n."""
    import torch
    from pymoto_gb300.mma import MMAUpdate
    from oracle.mma import MMAOracle
    shape = (96, 48, 48) if args.shape is None else tuple(int(v) for v in args.shape.split("x"))
    n = int(np.prod([max(v, 1) for v in shape]))
    rng = np.random.default_rng(7)
    x0 = rng.uniform(0.2, 0.8, n)
    dg = np.vstack([-rng.uniform(0.0, 2.0, n) * 10.0 / n, np.full(n, 1.0 / n)])
    g = np.array([10.0, float(x0.mean() - 0.45)])
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()  # noqa: E731
    o = MMAOracle(n, 2, move=0.2)
    t0 = time.perf_counter()
    xo = o.step(x0, g, dg)
    t_cpu = time.perf_counter() - t0
    out = {"case": "mma", "n": n, "m": 1, "oracle_update_s": t_cpu, "oracle_newton_iterations": o.stats["newton"],
           "cpu_threads": os.cpu_count()}
    for variant, exact in (("fast", False), ("exact", True)):
        up = MMAUpdate(n, 2, 0.0, 1.0, move=0.2, exact=exact)
        x, gd, dgd = dev(x0), dev(g), dev(dg)
        first = None
        times, newton = [], []
        for k in range(7):
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            xn = up.step(x, gd, dgd)
            e1.record()
            torch.cuda.synchronize()
            if k == 0:
                first = xn.cpu().numpy()
            if k >= 2:
                times.append(e0.elapsed_time(e1) * 1e3)
                newton.append(up.stats["newton"])
            x = xn
        out[variant] = {"update_us": float(np.mean(times)), "update_us_all": times, "newton_iterations": newton,
                        "max_abs_diff_first_update": float(np.abs(first - xo).max())}
    print(json.dumps(out))


def mma_run_case(args):
    """The 96x48x48 MMA workload: a fixed number of MMA iterations (--mma-iters, default 100) of the compliance
    cantilever with a volume constraint of 0.5, every module, the sensitivities and the MMA update on the device,
    for three solver arms: mixed with the learned warm start pretrained on --pretrain (default 256) seeded
    smoothed-noise fields (Gaussian-smoothed U(0,1), sigma 4 elements, mapped to [1e-3, 1]) and trained online,
    mixed without it, and plain FP64.  Objective Scaling(100) of the compliance, constraint 10 (mean(xf) - 0.5),
    MMA2007 with move 0.2, x0 = 0.5.  Whole-loop times with CUDA events (synchronised each iteration, as the
    optimizer reads its responses), printed as one JSON line."""
    import torch
    import pymoto_gb300 as pg
    from scipy.ndimage import gaussian_filter
    shape = (96, 48, 48) if args.shape is None else tuple(int(v) for v in args.shape.split("x"))
    iters = args.mma_iters
    npre = args.pretrain
    o = DesignRun.opts
    out = {"case": "mma_run", "shape": list(shape), "iterations": iters, "pretrain_fields": npre, "arms": {}}
    for arm in ("mixed_learned", "mixed", "plain_fp64"):
        d = pg.VoxelDomain(*shape)
        bc, f = cantilever(shape)
        fd = torch.from_numpy(f).cuda()
        sx = pg.Signal("x", torch.full((d.nel,), 0.5, dtype=torch.float64, device="cuda"))
        mixed = arm.startswith("mixed")
        ws = None
        with pg.Network() as fn:
            xf = pg.FilterConv(d, radius=RADIUS)(sx)
            xs = pg.SIMP(xmin=XMIN, penal=PENAL)(xf)
            K = pg.AssembleStiffness(d, bc=bc, sensitivity_precision="mixed" if mixed else "fp64")(xs)
            if mixed:
                mgs = pg.GeometricMultigrid.hierarchy(d, levels=o["levels"], smooth_steps=o["cheb_degree"],
                                                      precision="fp32", coarse_smooth_steps=o["cheb_coarse_degree"],
                                                      smoother="chebyshev", cheb_ratio=o["cheb_ratio"],
                                                      coarse_lag=o["coarse_lag"])
                if arm == "mixed_learned":
                    from pymoto_gb300.learned import LearnedWarmStart
                    ws = LearnedWarmStart(shape, stride=o["learned_stride"], capacity=8,
                                          train_steps=o["learned_train_steps"], lr=o["learned_lr"], seed=1234,
                                          history=o["learned_history"], train_every=o["learned_train_every"],
                                          gate=o["learned_gate"], gate_skip=o["learned_gate_skip"])
                solver = pg.MixedPrecisionCG(preconditioner=mgs[0], tol=TOL, m=o["m"], inner_iters=o["inner_iters"],
                                             inner_tol=o["inner_tol"], warm_start=ws, verify_residual=False)
            else:
                mgs = pg.GeometricMultigrid.hierarchy(d, levels=o["levels"], smoother_w=OMEGA,
                                                      smooth_steps=o["sweeps"])
                solver = pg.CG(preconditioner=mgs[0], tol=TOL)
            u = pg.LinSolve(hermitian=True, symmetric=True, solver=solver)(K, fd)
            c = pg.EinSum("i,i->")(u, fd)
            g0 = pg.Scaling(scaling=100.0)(c)
            g1 = pg.Scaling(scaling=5.0, maxval=0.5 * d.nel)(pg.EinSum("i->")(xf))
        t_pre = 0.0
        if ws is not None and npre > 0:
            rng = np.random.default_rng(2024)
            t0 = time.perf_counter()
            for _ in range(npre):
                nz = max(shape[2], 1)
                field = gaussian_filter(rng.uniform(0.0, 1.0, (nz, shape[1], shape[0])), sigma=4.0)
                field = (field - field.min()) / max(field.max() - field.min(), 1e-300)
                sx.state = torch.from_numpy(1e-3 + (1.0 - 1e-3) * field.ravel()).cuda()
                fn.response()
            torch.cuda.synchronize()
            t_pre = time.perf_counter() - t0
            sx.state = torch.full((d.nel,), 0.5, dtype=torch.float64, device="cuda")
            fn.response()
        mma = pg.MMA(sx, [g0, g1], fn, move=0.2, verbosity=0)
        xval = mma.x
        # one untimed sensitivity pass: first uses of library kernels (module loading) stay out of the timing
        fn.reset()
        g0.sensitivity = 1.0
        fn.sensitivity()
        fn.reset()
        torch.cuda.synchronize()
        hist, solves = [], []
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(iters):
            xnew, gk, _ = mma.step(x=xval)
            hist.append(gk.cpu().numpy().tolist())
            solves.append(solver.iterations)
            xval = xnew
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / iters
        out["arms"][arm] = {"design_it_per_s": 1e3 / ms, "ms_per_iteration": ms,
                            "solver_iterations_mean": float(np.mean(solves)), "g_first": hist[0], "g_last": hist[-1],
                            "mean_x_last": float(xval.mean().item()), "pretrain_s": t_pre}
    print(json.dumps(out))


def main():
    args = parse()
    if args.case == "operator":
        operator_case(args)
        return
    if args.case == "mma":
        mma_case(args)
        return
    if args.case == "mma_run":
        mma_run_case(args)
        return
    if args.case == "poisson":
        poisson_case(args)
        return
    rank, world, local_rank = dist_info()
    threads = os.cpu_count() or 1
    if args.impl == "reference":
        if rank != 0:
            return
        shape = SHAPE if args.shape is None else tuple(int(v) for v in args.shape.split("x"))
        times, L = cpu_reference_sample(shape, warm_steps=max(1, args.steps), warmup=args.warmup,
                                        seed=replica_seed(0))
        per = statistics.mean(times)
        line = {"metric": METRIC, "value": 1.0 / per, "unit": "design it/s", "impl": "reference", "n_gpus": args.gpus,
                "steps": len(times), "warmup": max(1, args.warmup), "ms_per_step": per * 1e3,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                "data": "synthetic (seeded U(1e-3,1) density, the GPU arms' seed)",
                "config": {"workload": f"3D cantilever hex8 {shape[0]}x{shape[1]}x{shape[2]}, FilterConv r=2.5, "
                                       f"SIMP p=3, CG+GMG {REF_LEVELS} levels (SuperLU coarsest), tol 1e-6, OC"},
                "cpu_baseline": {"value": 1.0 / per, "unit": "design it/s", "cores": threads, "kind": "port",
                                 "sample": f"design iterations {max(1, args.warmup) + 1}..{max(1, args.warmup) + len(times)} "
                                           f"of the run (the same designs the GPU arms time), after "
                                           f"{max(1, args.warmup)} untimed; numpy/scipy restatement of pyMOTO's path "
                                           f"(assembly by add.at, SpGEMM Galerkin, SuperLU coarsest, CG), "
                                           f"OMP/OPENBLAS threads = {os.environ.get('OMP_NUM_THREADS')}"},
                "e2e": {"value": 1.0 / per, "unit": "design it/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
                "cg_iterations": L.solver.cg_iterations}
        print(json.dumps(line))
        return

    import torch
    if world > 1:
        torch.distributed.init_process_group("nccl")
    m = measure_gb300(args, rank, world, local_rank)
    if m is None:
        return
    if rank == 0:
        shape = m["shape"]
        R = m["results"]
        steps = args.steps
        H = headline_arm(R)
        val_head = aggregate_rate(world, steps, R[H]["total_ms"] / 1e3)
        val_mixed = aggregate_rate(world, steps, R["mixed"]["total_ms"] / 1e3) if "mixed" in R else None
        val_plain = aggregate_rate(world, steps, R["plain_fp64"]["total_ms"] / 1e3) if "plain_fp64" in R else None
        # rooflines of the level-0 operator kernels, timed live after the timed region (kernel_rooflines)
        K = m["kernels"]
        sel = K["selected"]
        kdesc = {"fma": "ebe_apply_fma_kernel<residual> (FP32 operator, FP32 FMAs on the CUDA cores, one thread per "
                        "node column)",
                 "tcgen05": "ebe_apply_tc_kernel<residual> (FP32 operator, 3xTF32 tcgen05.mma, A read by the tensor "
                            "core from the staged node layers, accumulators in TMEM)"}
        fp32_peak = 2 * 128 * torch.cuda.get_device_properties(0).multi_processor_count * \
            m["peaks"].get("sm_max_mhz", 2070.0) * 1e6 / 1e12            # 128 FP32 FMA/clk/SM nominal
        tf32_peak = m["peaks"].get("bf16_tflops", 1900.0) / 2.0       # dense TF32 runs at half the BF16 rate

        def op_roofline(kind):
            km = K[f"ebe_apply_{kind}_residual_f32"]
            achieved = km["bytes"] / km["s"] / 1e9
            r = {"bound": "hbm", "kernel": kdesc[kind] + ", grid %s" % "x".join(map(str, shape)),
                 "achieved": achieved, "peak": m["hbm_peak"], "unit": "GB/s", "frac": achieved / m["hbm_peak"],
                 "traffic": NCU_TRAFFIC_PER_LAUNCH.get(f"ebe_apply_{kind}_residual_f32"),
                 "bytes_per_launch": km["bytes"], "avg_launch_us": km["s"] * 1e6, "peak_source": m["peak_src"],
                 "fp32_tflops": km["flops"] / km["s"] / 1e12,
                 "fp32_frac_of_nominal": km["flops"] / km["s"] / 1e12 / fp32_peak}
            if kind == "tcgen05":
                r["tensor_tflops"] = 3 * km["flops"] / km["s"] / 1e12
                r["tensor_frac_of_tf32"] = r["tensor_tflops"] / tf32_peak
            return r

        roofline = op_roofline(sel)
        roofline.update({"launches_per_step": "3 per inner FP32 PCG iteration (matvec, V-cycle residual, Chebyshev "
                                              "step)",
                         "note": "one launch at a time after a 256 MB L2 flush, CUDA events on the launching stream"})
        roofline_alt = {k: op_roofline(k) for k in kdesc if k != sel}
        ks = K["stencil_apply_f64_matvec"]
        sms = torch.cuda.get_device_properties(0).multi_processor_count
        fp64_peak = 2 * 2 * sms * m["peaks"].get("sm_max_mhz", 2070.0) * 1e6 / 1e12   # 2 DFMA/clk/SM nominal
        roofline_fp64 = {"bound": "fp64", "kernel": "stencil_apply_kernel<double> (outer FP64 operator)",
                         "achieved": ks["flops"] / ks["s"] / 1e12, "peak": fp64_peak, "unit": "TFLOP/s",
                         "frac": ks["flops"] / ks["s"] / 1e12 / fp64_peak, "avg_launch_us": ks["s"] * 1e6,
                         "hbm_gbs": ks["bytes"] / ks["s"] / 1e9, "peak_source": "nominal 2 FP64 FMA/clk/SM x SMs x "
                                                                                "max SM clock"}
        cpu = None
        parity_oracle = None
        if not args.no_cpu_baseline and world == 1:
            times, L = cpu_reference_sample(shape, warm_steps=args.cpu_steps, warmup=1, seed=replica_seed(0))
            cpu = {"value": 1.0 / statistics.median(times), "unit": "design it/s", "cores": os.cpu_count(),
                   "kind": "port", "median_s": statistics.median(times), "times_s": times,
                   "sample": f"median of {len(times)} warm design iterations (iterations 2..{len(times) + 1} of the "
                             f"same seeded workload, after 1 cold one) with the numpy/scipy restatement of pyMOTO's "
                             f"path, 4-level CG+GMG, OMP/OPENBLAS threads = {os.environ.get('OMP_NUM_THREADS')}"}
            if m["design1"] is not None:
                # the oracle as the checker: pyMOTO's FP64 CG + GMG to a relative residual of 1e-12 on the first
                # design, against both GPU solvers' solutions of it
                import oracle
                t0 = time.perf_counter()
                ref = oracle.fp64_cg_reference(shape, m["design1"]["x"], radius=RADIUS, levels=REF_LEVELS, w=OMEGA,
                                               smooth_steps=SWEEPS, tol=1e-12)
                parity_oracle = {"design": "the first design of the timed runs (seeded U(1e-3, 1))",
                                 "oracle": f"FP64 CG + GMG ({REF_LEVELS} levels) to recursive relative residual 1e-12, "
                                           f"{ref['iterations']} iterations, true relative residual "
                                           f"{ref['residual']:.3e}, {time.perf_counter() - t0:.1f} s on the host",
                                 "fp64": parity_errors(m["design1"]["fp64"], ref),
                                 "mixed": parity_errors(m["design1"]["mixed"], ref)}
        e2e_val = aggregate_rate(world, steps, m["e2e_total_s"])
        launches = R[H]["probe"].launches
        line = {"metric": METRIC, "value": val_head, "unit": "design it/s", "n_gpus": world, "steps": steps,
                "warmup": args.warmup, "ms_per_step": R[H]["total_ms"] / steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64/f32",
                "data": "synthetic (seeded U(1e-3,1) initial density, replicas seeded per rank)",
                "config": {"workload": f"3D cantilever hex8 {shape[0]}x{shape[1]}x{shape[2]} "
                                       f"({3 * (shape[0] + 1) * (shape[1] + 1) * (shape[2] + 1)} dofs), FilterConv "
                                       f"r=2.5, SIMP p=3, OC move 0.2, rel. residual 1e-6",
                           "solver": f"FP64 FCG({args.fcg_m}) preconditioned by {args.inner_iters} FP32 PCG "
                                     f"iterations on FP32 GMG {args.levels} levels (l1-Jacobi Chebyshev degree "
                                     f"{DesignRun.opts['cheb_degree']}/{DesignRun.opts['cheb_coarse_degree']} "
                                     f"fine/coarse), FP64 Cholesky coarsest with FP32 inverse"
                                     f"{' (previous inverse until the new one is ready)' if DesignRun.opts['coarse_lag'] else ''}"
                                     f"; plain arm: FP64 CG + FP64 GMG, damped Jacobi w=0.6, 2 sweeps, FP64 inverse",
                           "headline_arm": H, "learned_warm_start": H == "mixed_learned",
                           "learned_warm_start_note": "3-level BF16 conv net on the stride-4 voxels, trained on "
                                                      "the device every 4th solve; its prediction enters a "
                                                      "Rayleigh-Ritz initial guess with the previous solution, "
                                                      "skipped for 3 designs when it carried < 2 % of the guess's "
                                                      "energy (the deflation on its span, learned_cc, is off: no "
                                                      "gain at this size); arms.mixed is the solver without it",
                           "parallelism": f"replicas x{world}", "l2": "flushed before every step (256 MB write)"},
                "arms": {arm: {"design_it_per_s": aggregate_rate(world, steps, R[arm]["total_ms"] / 1e3),
                               "ms_per_step": R[arm]["total_ms"] / steps,
                               "solver_iterations": R[arm]["iters"], "true_rel_residual_last": R[arm]["true_residual"],
                               "compliance_last": R[arm]["compliance"]} for arm in R},
                "speedup_headline_vs_plain_fp64": val_head / val_plain if val_plain else None,
                "speedup_mixed_vs_plain_fp64": val_mixed / val_plain if (val_plain and val_mixed) else None,
                "parity": {"same_design_compliance_mixed": m["c_mixed"], "same_design_compliance_fp64_tol1e-11":
                           m["c_tight"], "rel_diff": abs(m["c_mixed"] - m["c_tight"]) / abs(m["c_tight"]),
                           "mixed_true_rel_residual": m["res_mixed_same_design"]},
                "parity_vs_oracle": parity_oracle,
                "roofline": roofline, "roofline_other_operator_kernels": roofline_alt,
                "roofline_fp64_stencil": roofline_fp64, "cpu_baseline": cpu,
                "e2e": {"value": e2e_val, "unit": "design it/s", "h2d_bytes_per_step": 8 * m["nel"],
                        "d2h_bytes_per_step": 8 * m["nel"] + 8, "arm": H,
                        "same_designs_as_value": m["e2e_same_designs"],
                        "note": "a second run of the headline arm from the same seed, the same warm-up, then the "
                                "same designs with the design vector copied host->device and the compliance and "
                                "new design device->host every step (pinned buffers), wall clock per step"},
                "gpu_launches": launches, "clocks": R[H]["clocks"]}
        if "breakdown" in m:
            print(json.dumps({"breakdown": {"|".join(map(str, k)): v for k, v in sorted(
                m["breakdown"].items(), key=lambda kv: -kv[1]["total_ms"])}}), file=sys.stderr)
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
