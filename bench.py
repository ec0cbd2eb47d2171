"""Benchmark of the GB300 hot path on the 160k-element hex8 J2 model (100x40x40 box).

Workload (one "step" = one load increment of the Newton driver: element loop, 3x3-block
assembly, Krylov solve, repeated until the reference's convergence test passes):
  C3D8 box 100x40x40 on 10x4x4, J2 [E=210000, nu=0.3, fy=250, H=1000], x=0 clamped,
  x=10 face pulled to u_x = 0.02 over 20 increments (maxInc 0.05).  The load history is
  advanced (untimed) into the plastic regime; every timed step re-solves the same
  plastic increment from the same committed state (the trial state is not accepted).
  Inputs are resident and larger than L2 (BSR system 159 MB FP32, element state 266 MB).

value     : load-step seconds with FGMRES(64) preconditioned by the smoothed-aggregation
            multigrid cycle (fused one-pass kernels per level) plus the learned message-passing
            correction when a validation solve shows that it makes the step faster (trained on
            pairs from the plain solves of the load history), FP32 inner iterations with FP64
            refinement to 1e-8
comparison: the same load step with block-Jacobi PCG (same system, same tolerance)
e2e       : the same as value through the public Python API with the step's inputs (U_n, dU)
            copied from pinned host memory and the results (U, P) read back every step
roofline  : the FGMRES product (the largest kernel of the step: FP32 sliced-ELL blocks, one
            launch per iteration), timed live with CUDA events; the fused fine post-smoothing and
            the fine residual (one launch each per iteration) beside it
cpu_baseline: the numpy oracle (restatement of the reference's CPU path) on a bounded sample

python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--nx 100 --ny 40 --nz 40]
"""

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

PROPS = [210000.0, 0.3, 250.0, 1000.0, 0.0, 0.0]
METRIC = "hex8 J2 load-step s: learned-FGMRES vs Jacobi-PCG @1e-8 resid; assembly GB/s"
# DRAM bytes (read + write) per launch of the fine-level kernels of the FGMRES solve on the
# 100x40x40 box (509,343 DOF, 4,406,941 blocks; the slices in their diagonal form), from one ncu
# capture of bench.py --profile --method fgmres
SWEEP_TRAFFIC_BYTES = 87.45e6
PRODUCT_TRAFFIC_BYTES = 176.73e6  # each slice split over 4 warps (170.52e6 with one warp per slice)
POST_TRAFFIC_BYTES = 95.23e6
# Newton iterations of the timed increment (13) of the 100x40x40 model: the same in the all-FP64
# and the mixed-precision GPU solves; the CPU arms charge this many element passes and solves
PCG_NEWTON_PER_STEP = 8
# Jacobi-CG iterations per sample step of the reference arm (timed on the full CPU system)
CG_SAMPLE = 20


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--nx", type=int, default=100)
    ap.add_argument("--ny", type=int, default=40)
    ap.add_argument("--nz", type=int, default=40)
    ap.add_argument("--increment", type=int, default=13, help="load increment re-solved in the timed steps")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-parity", action="store_true", help="skip the all-FP64 solve of the timed increment")
    ap.add_argument("--no-other-workloads", action="store_true",
                    help="skip the tied-box and cube-batch records nested in the headline line")
    ap.add_argument("--no-learned", action="store_true", help="FGMRES + multigrid without the learned correction")
    ap.add_argument("--no-learned-family", action="store_true",
                    help="skip the learned correction's cross-seed measurement on the seeded J2 family")
    ap.add_argument("--pcg-steps", type=int, default=2, help="timed steps of the Jacobi-PCG comparison")
    ap.add_argument("--restart", type=int, default=64, help="FGMRES restart length")
    ap.add_argument("--inner-rtol", type=float, default=1e-4,
                    help="relative tolerance of the first inner (FP32) solve of a system (the later ones: 1e-2 or "
                         "what the remaining target needs)")
    ap.add_argument("--precond-reuse", type=int, default=1,
                    help="Newton systems of an increment that reuse the coarse multigrid levels of its first one")
    ap.add_argument("--method", default="fgmres", choices=["pcg", "fgmres"], help="solver of --profile")
    ap.add_argument("--workload", default="box", choices=["box", "cubes", "tied"],
                    help="box: the 160k-element J2 box (default); cubes: 1024 independent J2 cubes in one batch; "
                         "tied: 60x30x30 NeoHookeWa box, hex20 | hex8 halves with a tied interface")
    ap.add_argument("--profile", action="store_true",
                    help="one assembly and one capped solve, for ncu captures of single kernels")
    ap.add_argument("--profile-learned", action="store_true",
                    help="with --profile: FGMRES with the learned correction enabled (untrained weights), 5 iterations")
    return ap.parse_args()


def multigrid_description(reuse=0):
    """The multigrid cycle as the library sets it up (its environment options, defaults otherwise)."""
    smoothed = os.environ.get("EF_AMG_SMOOTHED", "1") not in ("", "0")
    wl = int(os.environ.get("EF_AMG_WLEVELS", "0" if smoothed else "1"))
    sweeps = os.environ.get("EF_AMG_SWEEPS", "1" if smoothed else "2")
    pre, post = os.environ.get("EF_AMG_PRE", sweeps), os.environ.get("EF_AMG_POST", sweeps)
    kind = "smoothed-aggregation" if smoothed else "rigid-body aggregation"
    cycle = "V-cycle" if wl == 0 else ("W-cycle on level 1" if wl == 1 else f"W-cycle on levels 1-{wl}")
    lag = f", coarse levels built once per increment and reused by up to {reuse} Newton systems" if reuse else ""
    return f"{kind} multigrid, {cycle}, {pre}/{post} block-Jacobi sweeps{lag}"


def workload(a):
    return {
        "workload": f"hex8 J2 box {a.nx}x{a.ny}x{a.nz} (C3D8, 2x2x2 Gauss), pull 0.02 over 20 increments",
        "elements": a.nx * a.ny * a.nz,
        "dofs": 3 * (a.nx + 1) * (a.ny + 1) * (a.nz + 1),
        "material": "J2 E=210000 nu=0.3 fy=250 H=1000",
        "timed_increment": a.increment,
        "l2": "inputs larger than L2 (BSR system and element state resident, > 129 MB)",
    }


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    def __init__(self):
        self.samples = []
        self._stop = threading.Event()
        self._t = None

    def start(self):
        q = ("clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")  # fmt: skip

        def run():
            while not self._stop.is_set():
                try:
                    out = subprocess.run(["nvidia-smi", "-i", "0", f"--query-gpu={q}", "--format=csv,noheader,nounits"],
                                         capture_output=True, text=True, timeout=5).stdout.strip()  # fmt: skip
                    if out:
                        self.samples.append([x.strip() for x in out.split(",")])
                except Exception:
                    pass
                self._stop.wait(0.2)

        self._t = threading.Thread(target=run, daemon=True)
        self._t.start()

    def stop(self):
        self._stop.set()
        if self._t:
            self._t.join(timeout=10)
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4) if len(s) > 2 + i and s[2 + i] == "Active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}  # fmt: skip


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


def build_solver(a, linsolver, keFp64=False):
    from edelweissfe_gb300.mesh import box_mesh
    from edelweissfe_gb300.model import DirichletBC, ElementGroup, Model
    from edelweissfe_gb300.solver import NISTGPU

    lX, lY, lZ = 0.1 * a.nx, 0.1 * a.ny, 0.1 * a.nz
    m = box_mesh(a.nx, a.ny, a.nz, lX, lY, lZ)
    model = Model(m["coords"], [ElementGroup("C3D8", m["elements"], "vonmises", np.array(PROPS))])
    dirs = [DirichletBC(m["nodeSets"]["gen_left"], {0: 0.0, 1: 0.0, 2: 0.0}),
            DirichletBC(m["nodeSets"]["gen_right"], {0: 0.002 * lX})]  # fmt: skip
    return NISTGPU(model, dirs, linsolver=linsolver, keFp64=keFp64)


def fp64_parity(a, s, U_n, dU_n, target, prev, step, U_head, newton_head):
    """The timed increment solved again in all-FP64 arithmetic (FP64 element stiffness and
    system, FP64 block-Jacobi PCG to 1e-10) from the same committed state, U_n and dU: the
    headline solve's largest displacement and stress differences relative to it, and both
    Newton counts."""
    import torch

    from edelweissfe_gb300 import _lib
    from edelweissfe_gb300.solver import LinSolverOptions

    t0 = time.time()
    ref = build_solver(a, LinSolverOptions(method="pcg", mixed=False, rtol=1e-10, maxIter=200000), keFp64=True)
    try:
        nEl = a.nx * a.ny * a.nz
        gid_s, gid_r = s.groupIds[0], ref.groupIds[0]
        nQP, nState = ctypes_state_size(s, gid_s)
        committed = np.zeros((nEl, nQP, nState))
        _lib.check(s.lib.ef_get_state(s.ctx, gid_s, 0, committed.ctypes.data), "ef_get_state")
        _lib.check(ref.lib.ef_set_state(ref.ctx, gid_r, committed.ctypes.data), "ef_set_state")
        _lib.check(ref.lib.ef_set_dirichlet(ref.ctx, ref.dirIdxHost.ctypes.data, ref.dirIdxHost.size), "dir")
        U64, _, _, newton64 = ref.solveIncrement(U_n.clone(), dU_n.clone(), ref._vec(), target, prev, step)
        u64, uh = U64.cpu().numpy(), U_head.cpu().numpy()
        trial_s = np.zeros((nEl, nQP, nState))
        trial_r = np.zeros((nEl, nQP, nState))
        _lib.check(s.lib.ef_get_state(s.ctx, gid_s, 1, trial_s.ctypes.data), "ef_get_state")
        _lib.check(ref.lib.ef_get_state(ref.ctx, gid_r, 1, trial_r.ctypes.data), "ef_get_state")
        torch.cuda.synchronize()
        du = float(np.max(np.abs(uh - u64)) / np.max(np.abs(u64)))
        ds = float(np.max(np.abs(trial_s[..., :6] - trial_r[..., :6])) / np.max(np.abs(trial_r[..., :6])))
        return {"against": "all-FP64 solve of the same increment (FP64 stiffness, FP64 block-Jacobi PCG to 1e-10)",
                "max_rel_dU": du, "max_rel_dstress": ds, "newton_headline": int(newton_head),
                "newton_fp64": int(newton64), "newton_equal": int(newton_head) == int(newton64),
                "within_1e-6": du <= 1e-6, "wall_s": time.time() - t0}  # fmt: skip
    finally:
        del ref


def ctypes_state_size(s, gid):
    import ctypes

    nQP, nState = ctypes.c_int(), ctypes.c_int()
    s.lib.ef_get_state_size(s.ctx, gid, ctypes.byref(nQP), ctypes.byref(nState))
    return nQP.value, nState.value


def pcg_bytes_per_iteration(info, fp32=True):
    """Algorithmic DRAM bytes of one PCG iteration on the BSR(3x3) system."""
    s = 4 if fp32 else 8
    nb, nn, nd = info.nBlocks, info.nNodes, info.nDof
    spmv = nb * (9 * s + 4) + (nn + 1) * 4 + nd * s + nd * s  # values + columns + row pointers + p gather + q write
    update = nd * s * (2 + 2 + 1 + 1) + nn * 9 * s + nd  # x rw, r rw, q r, z w; block inverses; mask
    pupdate = nd * s * 3  # z r, p rw
    return spmv + update + pupdate


def assembly_bytes(info, nEl, fp32=True):
    """Algorithmic DRAM bytes of one assembly (element kernel + condensation + BSR scatter)."""
    s = 4 if fp32 else 8
    nQP = 8
    # node ids, state r/w, Ke blocks, Pe, geometry cache (dN/dx and w detJ per Gauss point, FP64), dU
    elem = nEl * (8 * 4 + nQP * 13 * 8 * 2 + 36 * 9 * s + 24 * 8 + nQP * 25 * 8) + info.nDof * 8
    cond = nEl * 24 * 8 + nEl * 8 * 8 + info.nDof * 8 * 2  # Pe read, map, P and F write
    scatter = nEl * 36 * 9 * s + nEl * 64 * 8 + info.nBlocks * (9 * s + 8)  # Ke read, map, BSR write
    return elem, cond, scatter


def learned_seeded_family(train=(0, 1, 2, 3), test=(4, 5), increments=14):
    """The learned correction on the seeded J2 family (per seed sigma_y ~ U[150,350],
    H ~ U[200,2000], nu ~ U[0.2,0.4]): trained on the Newton-iteration pairs of the `train` seeds'
    load histories (one context, one box per seed), then the load history of the unseen `test`
    seeds with and without it, over the block-Jacobi base (16x8x8 boxes: FGMRES + block Jacobi
    stalls on the plastic systems of larger boxes) and over the multigrid base (40x16x16 boxes)."""
    from edelweissfe_gb300.learned import evaluate_on_seeds, train_across_seeds

    out = {"increments": increments}
    for base, dims in (("jacobi", (16, 8, 8)), ("multigrid", (40, 16, 16))):
        try:
            params, scales, rec = train_across_seeds(list(train), dims, increments, base=base, epochs=100)
            ev = evaluate_on_seeds(list(test), dims, increments, params, scales, base=base)
            out[base] = {"box": "x".join(map(str, dims)), "train": rec, "unseen": ev}
        except Exception as ex:  # reported, not fatal to the bench
            out[base] = {"error": f"{type(ex).__name__}: {ex}"}
    return out


def run_ours(a):
    import torch

    from edelweissfe_gb300 import _lib
    from edelweissfe_gb300 import build as b
    from edelweissfe_gb300.solver import AdaptiveTimeStepper, LinSolverOptions, Step

    b.build()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    dev = torch.device("cuda", local)
    t0 = time.time()
    s = build_solver(a, LinSolverOptions(method="fgmres", rtol=1e-8, restart=a.restart, innerRtol=a.inner_rtol,
                                         precondReuse=a.precond_reuse))  # fmt: skip
    setup_s = time.time() - t0
    info = s.info
    lib = s.lib
    stream = torch.cuda.current_stream()
    step = Step(maxInc=0.05, minInc=1e-6, maxIter=25)
    _lib.check(lib.ef_set_dirichlet(s.ctx, s.dirIdxHost.ctypes.data, s.dirIdxHost.size), "dir")
    learned = not a.no_learned
    if learned:
        s.initLearnedPreconditioner(seed=0, maxSamples=64)
        s.collectTrainingPairs(every=20, maxPerSolve=12, kind="iterates")

    # advance the load history (untimed, FGMRES without the learned stage, collecting pairs) up to
    # the increment that the steps re-solve
    U, dU, P = s._vec(), s._vec(), s._vec()
    prev = None
    stepper = AdaptiveTimeStepper(0.0, 1.0, step.startInc, step.maxInc, step.minInc, step.maxNumInc)
    history, target = [], None
    t0 = time.time()
    for ts in stepper.generateTimeStep():
        if ts.number == a.increment:
            target = ts
            break
        U, dU, P, it = s.solveIncrement(U, dU, P, ts, prev, step)
        _lib.check(lib.ef_accept_state(s.ctx), "accept")
        history.append(it)
        prev = ts
    history_s = time.time() - t0
    U_n, dU_n = U.clone(), dU.clone()

    def one_step():
        s.krylovIterations.clear()
        _, _, _, it = s.solveIncrement(U_n, dU_n.clone(), s._vec(), target, prev, step)
        return it

    def timed(n):
        torch.cuda.synchronize()
        t = time.perf_counter()
        its = [one_step() for _ in range(n)]
        torch.cuda.synchronize()
        return (time.perf_counter() - t) / n, its, sum(s.krylovIterations)

    learned_info = None
    if learned:
        s.collectTrainingPairs(0, 0)
        t0 = time.time()
        lf, ll = s.trainLearnedPreconditioner(epochs=20, lr=3e-4, norm="energy")
        torch.cuda.synchronize()
        train_s = time.time() - t0
        # validation on the timed increment (these solves are part of the warm-up)
        s.enableLearnedPreconditioner(False)
        off_s, _, off_k = timed(1)
        s.enableLearnedPreconditioner(True)
        timed(1)
        on_s, _, on_k = timed(1)
        keep = on_s < off_s
        s.enableLearnedPreconditioner(keep)
        learned_info = {"pairs": s.numTrainingPairs(), "epochs": 20, "loss": "energy", "loss_first": lf,
                        "loss_last": ll, "train_s": train_s,
                        "validation": {"on_s": on_s, "off_s": off_s, "on_krylov": on_k, "off_krylov": off_k},
                        "enabled": keep}  # fmt: skip

    for _ in range(a.warmup):
        one_step()
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    clocks = ClockSampler()
    clocks.start()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    newton, krylov = [], []
    torch.cuda.synchronize()
    l0 = lib.ef_kernel_launches()
    e0.record(stream)
    for _ in range(a.steps):
        newton.append(one_step())
        krylov.append(sum(s.krylovIterations))
    e1.record(stream)
    torch.cuda.synchronize()
    launches = lib.ef_kernel_launches() - l0
    clk = clocks.stop()
    t_step = e0.elapsed_time(e1) / 1e3 / a.steps
    if world > 1:
        t = torch.tensor([t_step], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        t_step = float(t.item())

    def profiled_step():
        infos = []
        orig = s.linearSolve

        def wrapped(R):
            x = orig(R)
            i = s.lastSolveInfo
            infos.append((i.kernelMs, i.iterations, i.kernelLaunches, i.spmvMs, i.spmvLaunches, i.precondMs,
                          i.orthoMs, i.reorths, i.refinements, 1, i.setupMs))
            return x

        s.linsolver.profile = True
        s.linearSolve = wrapped
        try:
            one_step()
        finally:
            s.linearSolve = orig
            s.linsolver.profile = False
        return [sum(x[i] for x in infos) for i in range(11)]

    fg_kms, fg_it, _, sp_ms, sp_n, pre_ms, orth_ms, n_reorth, n_refine, n_solves, setup_ms = profiled_step()

    def phase_step():
        # wall time of each Newton-loop phase over one step (synchronised around each call, so the
        # phases do not overlap; the rest of the step is the driver's own work)
        names = ("computeElements", "assembleStiffnessCSR", "newtonResidual", "linearSolve")
        acc = {k: 0.0 for k in names}
        origs = {k: getattr(s, k) for k in names}

        def timed_call(k):
            def f(*args, **kw):
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                out = origs[k](*args, **kw)
                torch.cuda.synchronize()
                acc[k] += time.perf_counter() - t0
                return out

            return f

        for k in names:
            setattr(s, k, timed_call(k))
        try:
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            one_step()
            torch.cuda.synchronize()
            total = time.perf_counter() - t0
        finally:
            for k in names:
                setattr(s, k, origs[k])
        out = {k: 1e3 * v for k, v in acc.items()}
        out["step"] = 1e3 * total
        out["rest"] = out["step"] - sum(out[k] for k in names)
        return out

    phase_ms = phase_step()
    # the fine-level kernels timed live on the timed increment's last system (CUDA events, same stream)
    import ctypes

    fk_ms, fk_bytes = (ctypes.c_double * 3)(), (ctypes.c_double * 3)()
    fk_ok = lib.ef_fine_kernel_profile(s.ctx, 50, fk_ms, fk_bytes, stream.cuda_stream) == _lib.EF_OK

    # comparison arm: block-Jacobi PCG on the same load step
    s.linsolver.method = "pcg"
    if learned:
        s.enableLearnedPreconditioner(False)
    one_step()
    pcg_s, pcg_newton, pcg_k = timed(max(1, a.pcg_steps))
    pcg_kms, pcg_it = profiled_step()[:2]
    s.linsolver.method = "fgmres"
    if learned_info and learned_info["enabled"]:
        s.enableLearnedPreconditioner(True)

    # assembly timing: element kernel + condensation + BSR scatter on resident inputs
    t2 = np.array([target.stepTime, target.totalTime])
    Pv, Fv = s._vec(), s._vec()
    times = {"elements": [], "assemble": []}
    for rep in range(6):
        ea, eb, ec = (torch.cuda.Event(enable_timing=True) for _ in range(3))
        ea.record(stream)
        _lib.check(lib.ef_compute_elements(s.ctx, U_n.data_ptr(), dU_n.data_ptr(), t2.ctypes.data,
                                           target.timeIncrement, Pv.data_ptr(), Fv.data_ptr(), stream.cuda_stream),
                   "ce")  # fmt: skip
        eb.record(stream)
        _lib.check(lib.ef_assemble_bsr(s.ctx, stream.cuda_stream), "bsr")
        ec.record(stream)
        torch.cuda.synchronize()
        if rep >= 2:
            times["elements"].append(ea.elapsed_time(eb))
            times["assemble"].append(eb.elapsed_time(ec))
    lib.ef_element_status(s.ctx, stream.cuda_stream, None)
    nEl = a.nx * a.ny * a.nz
    b_elem, b_cond, b_scat = assembly_bytes(info, nEl)
    t_el = float(np.median(times["elements"])) * 1e-3
    t_as = float(np.median(times["assemble"])) * 1e-3
    asm_gbs = (b_elem + b_cond + b_scat) / (t_el + t_as) / 1e9

    # e2e through the public API: host inputs -> device, load step, results -> host
    hU = U_n.cpu().pin_memory()
    hdU = dU_n.cpu().pin_memory()
    outU = torch.empty(s.nDof, dtype=torch.float64).pin_memory()
    outP = torch.empty(s.nDof, dtype=torch.float64).pin_memory()
    e2e_steps = max(1, min(a.steps, 3))
    torch.cuda.synchronize()
    f0 = torch.cuda.Event(enable_timing=True)
    f1 = torch.cuda.Event(enable_timing=True)
    f0.record(stream)
    for _ in range(e2e_steps):
        Ud = hU.to(dev, non_blocking=True)
        dUd = hdU.to(dev, non_blocking=True)
        Unp, _, Pd, _ = s.solveIncrement(Ud, dUd, s._vec(), target, prev, step)
        outU.copy_(Unp, non_blocking=True)
        outP.copy_(Pd, non_blocking=True)
    f1.record(stream)
    torch.cuda.synchronize()
    e2e_s = f0.elapsed_time(f1) / 1e3 / e2e_steps

    # parity of the timed increment at full size: the headline solve against an all-FP64 one
    parity = None
    if not a.no_parity:
        Uh, _, _, nh = s.solveIncrement(U_n, dU_n.clone(), s._vec(), target, prev, step)
        parity = fp64_parity(a, s, U_n, dU_n, target, prev, step, Uh, nh)

    # the learned correction trained across seeds of the J2 family and used on unseen seeds
    if learned and not a.no_learned_family:
        learned_info["seeded_family"] = learned_seeded_family()

    # the other two workloads of the suite, each in its own context: the tied hex20 | hex8 box and
    # the batch of 1024 cubes (one whole load history); their records are nested in this line
    others = None
    if not a.no_other_workloads and rank == 0:
        others = {}
        for key, fn, args in (("tied", measure_tied, (3, 3)), ("cubes", measure_cubes, (1, 1))):
            try:
                others[key] = fn(*args)
            except Exception as ex:  # reported, not fatal to the headline
                others[key] = {"error": f"{type(ex).__name__}: {ex}"}
            torch.cuda.synchronize()

    peaks, peak_kind = measured_peaks()
    full = a.nx * a.ny * a.nz == 160000
    roofline = None
    if fk_ok:
        def entry(k, kernel, traffic):
            gbs = fk_bytes[k] / (fk_ms[k] * 1e-3) / 1e9
            return {"kernel": kernel, "achieved": gbs, "frac": gbs / peaks["hbm_gbs"], "bytes_per_launch": fk_bytes[k],
                    "avg_launch_ms": fk_ms[k], "traffic": traffic if full else None}

        # the dominant kernel of the load step: the FGMRES product (one launch per iteration, the
        # largest); the fused post-smoothing and the fine residual (one launch each per iteration) beside
        roofline = entry(1, "sell_spmv3_kernel (FGMRES product K z, FP32 sliced-ELL in its diagonal form: "
                            "columns computed from 27 node offsets; one launch per iteration)",
                         PRODUCT_TRAFFIC_BYTES)
        roofline.update({"bound": "hbm", "peak": peaks["hbm_gbs"], "peak_kind": peak_kind, "unit": "GB/s",
                         "traffic_source": "ncu (dram__bytes_read.sum + dram__bytes_write.sum per launch) of "
                                           "bench.py --profile --method fgmres",
                         "timing": "CUDA events, 50 back-to-back launches on the timed increment's last system"})
        if sp_n and sp_ms > 0:
            # the product's own launches inside the solve: CUDA events around each one on the solve's
            # stream, over one profiled replay of the timed increment
            in_ms = sp_ms / sp_n
            gbs = fk_bytes[1] / (in_ms * 1e-3) / 1e9
            roofline.update({"back_to_back_ms": roofline["avg_launch_ms"], "back_to_back_frac": roofline["frac"],
                             "avg_launch_ms": in_ms, "achieved": gbs, "frac": gbs / peaks["hbm_gbs"],
                             "timing": f"CUDA events around each of the {int(sp_n)} product launches of one profiled "
                                       "replay of the timed increment (the solve's stream); back_to_back_*: 50 "
                                       "launches in a row on its last system"})
        if fk_ms[2] > 0:
            roofline["second"] = entry(2, "sa_post_fused_kernel (fine prolongation + post-smoothing x = w D^-1 (r + t)"
                                          " + C e, C in BF16; 50 back-to-back launches)", POST_TRAFFIC_BYTES)
        roofline["third"] = entry(0, "sell_level3_bf16_kernel (fine residual t = r - w K M D^-1 r, BF16 "
                                     "sliced-ELL, diagonal form; 50 back-to-back launches)", SWEEP_TRAFFIC_BYTES)
    pcg_bpi = pcg_bytes_per_iteration(info)
    pcg_gbs = pcg_bpi * pcg_it / (pcg_kms * 1e-3) / 1e9 if pcg_kms > 0 else None
    cpu = None
    if rank == 0 and not a.no_cpu_baseline:
        cpu = cpu_baseline(a, newton_per_step=PCG_NEWTON_PER_STEP, procs=1)
    fg_k = float(np.mean(krylov))
    if learned_info and learned_info["enabled"]:
        stage = "learned correction kept"
    elif learned_info:
        stage = "learned correction trained, dropped by the validation solve"
    else:
        stage = "no learned correction"
    line = {
        "metric": METRIC,
        "value": t_step,
        "unit": "s",
        "n_gpus": world,
        "steps": a.steps,
        "warmup": a.warmup,
        "ms_per_step": t_step * 1e3,
        "higher_is_better": False,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64 residual/return map, f32 stiffness + Krylov inner, f64 refinement",
        "data": "synthetic (structured box mesh, seeded parameters)",
        "config": workload(a),
        "solver": f"FGMRES({a.restart}) + {multigrid_description(a.precond_reuse)} ({stage})",
        "newton_iterations_per_step": newton,
        "krylov_iterations_per_step": krylov,
        "comparison": {"jacobi_pcg_step_s": pcg_s, "speedup_vs_jacobi_pcg": pcg_s / t_step,
                       "jacobi_pcg_krylov_per_step": pcg_k, "fgmres_krylov_per_step": fg_k,
                       "krylov_ratio": pcg_k / fg_k if fg_k else None, "jacobi_pcg_newton": pcg_newton,
                       "jacobi_pcg_kernel_GBps": pcg_gbs,
                       "jacobi_pcg_frac_hbm": pcg_gbs / peaks["hbm_gbs"] if pcg_gbs else None},
        "learned": learned_info,
        "assembly": {"elements_ms": t_el * 1e3, "bsr_scatter_ms": t_as * 1e3, "GBps": asm_gbs,
                     "frac_hbm": asm_gbs / peaks["hbm_gbs"], "bytes": b_elem + b_cond + b_scat,
                     "elements_per_s": nEl / (t_el + t_as)},
        "phase_ms": phase_ms,
        "fgmres_profile": {"iterations": fg_it, "kernel_ms": fg_kms,
                           "ms_per_iteration": fg_kms / fg_it if fg_it else None,
                           "precond_ms_per_iteration": pre_ms / fg_it if fg_it else None,
                           "spmv_ms_per_iteration": sp_ms / fg_it if fg_it else None,
                           "ortho_ms_per_iteration": orth_ms / fg_it if fg_it else None,
                           "reorthogonalised_columns": int(n_reorth), "solves": int(n_solves),
                           "refinement_sweeps": int(n_refine), "restart": a.restart, "inner_rtol": a.inner_rtol,
                           "refine_floor": float(os.environ.get("EF_REFINE_FLOOR", "1e-2")),
                           "preconditioner_setup_ms": setup_ms},
        "dof_iterations_per_s": info.nDof * fg_it / (fg_kms * 1e-3) if fg_kms > 0 else None,
        "setup_s": setup_s,
        "history_s": history_s,
        "e2e": {"value": e2e_s, "unit": "s", "h2d_bytes_per_step": 2 * 8 * s.nDof, "d2h_bytes_per_step": 2 * 8 * s.nDof},
        "gpu_launches": int(launches),
        "roofline": roofline,
        "clocks": clk,
        "cpu_baseline": cpu,
        "parity": parity,
        "other_workloads": others,
        "history_newton": history,
    }  # fmt: skip
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def run_cubes(a):
    """1024 independent J2 hex8 cubes (edge n ~ U{4..16}, random sigma_y, H, nu per cube; base
    clamped, top pulled by 1 % in 10 increments): one step = the whole load history of the batch."""
    from edelweissfe_gb300 import build as b

    b.build()
    print(json.dumps(measure_cubes(a.steps, a.warmup)), flush=True)


def measure_cubes(steps, warmup):
    """The cube batch's JSON record (see run_cubes)."""
    import torch

    from edelweissfe_gb300.batch import BatchNISTGPU, cube_batch_spec
    from edelweissfe_gb300.solver import Step

    spec = cube_batch_spec(1024, 0)
    step = Step(maxInc=0.1, minInc=1e-6, maxIter=25)
    s = BatchNISTGPU(spec)
    for _ in range(max(1, warmup)):
        s.problemHistory.clear()
        s.krylovPerProblem[:] = 0
        s.solveStepBatch(step)
    clocks = ClockSampler()
    clocks.start()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    l0 = s.lib.ef_kernel_launches()
    e0.record()
    for _ in range(steps):
        s.problemHistory.clear()
        s.krylovPerProblem[:] = 0
        s.solveStepBatch(step)
    e1.record()
    torch.cuda.synchronize()
    launches = s.lib.ef_kernel_launches() - l0
    clk = clocks.stop()
    t = e0.elapsed_time(e1) / 1e3 / steps
    # batched-PCG roofline from one eager profiled run: bytes per problem-iteration = its blocks
    # (72 B values + 4 B column) + row pointers + 10 vector passes of its DOFs
    prof = BatchNISTGPU(spec, graph=False, tile=s.tile)
    prof.profile = True
    prof.solveStepBatch(step)
    nodes = np.diff(prof.nodePtr)
    info = prof.info
    rowBlocks = info.nBlocks / info.nNodes
    bytes_per_it = nodes * (rowBlocks * 76 + 4 + 3 * 8 * 10)
    total_bytes = float((prof.krylovPerProblem * bytes_per_it).sum())
    solve_s = sum(prof.solveMs) / 1e3
    peaks, peak_kind = measured_peaks()
    achieved = total_bytes / solve_s / 1e9
    hist = np.array([it for _, it in s.problemHistory])
    nEl = int(s.nElProb.sum())
    line = {
        "metric": "batched J2 cubes: load-history s (1024 cubes, 10 increments)",
        "value": t, "unit": "s", "n_gpus": 1, "steps": steps, "warmup": warmup, "ms_per_step": t * 1e3,
        "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64 (state, stiffness, PCG)", "data": "synthetic (seeded cube sizes and materials)",
        "config": {"workload": "1024 J2 hex8 cubes, n ~ U{4..16}, sigma_y ~ U[150,350], H ~ U[200,2000], "
                               "nu ~ U[0.2,0.4] (seed 0), base clamped, 1 % axial strain in 10 increments",
                   "elements": nEl, "dofs": int(s.nDof)},
        "newton_iterations_max_per_increment": hist.max(axis=1).tolist(),
        "krylov_iterations_total": int(s.krylovPerProblem.sum()),
        "tile": s.tile_shapes()[s.tile], "autotune_ms": s.tuning,
        "elements_per_s": nEl * int(hist.max(axis=1).sum()) / t,
        "dof_iterations_per_s": float((prof.krylovPerProblem * 3 * nodes).sum()) / solve_s,
        "gpu_launches": int(launches),
        "roofline": {"bound": "hbm", "kernel": "batched_pcg_kernel", "achieved": achieved, "peak": peaks["hbm_gbs"],
                     "peak_kind": peak_kind, "unit": "GB/s", "frac": achieved / peaks["hbm_gbs"], "traffic": None,
                     "solve_s": solve_s, "bytes": total_bytes},
        "clocks": clk,
    }  # fmt: skip
    return line


def run_tied(a):
    """60x30x30 box (h = 1/30): x < 30 C3D20TL, x >= 30 C3D8TL, NeoHookeWa [80, 200], tied
    interface, x = 0 clamped, x = 60 face compressed to 30 % over 40 increments.  A step is one
    load increment (all Newton iterations, state accepted); warm-up increments run first."""
    from edelweissfe_gb300 import build as b

    b.build()
    print(json.dumps(measure_tied(a.steps, a.warmup)), flush=True)


def measure_tied(steps, warmup):
    """The tied box's JSON record (see run_tied)."""
    import torch

    from edelweissfe_gb300 import _lib
    from edelweissfe_gb300.mesh import tied_box_mesh
    from edelweissfe_gb300.model import DirichletBC, ElementGroup, Model
    from edelweissfe_gb300.solver import AdaptiveTimeStepper, LinSolverOptions, NISTGPU, Step

    h = 1.0 / 30.0
    m = tied_box_mesh(30, 30, 30, 30, 30 * h, 30 * h, 30 * h, 30 * h)
    p = np.array([80.0, 200.0])
    model = Model(m["coords"], [ElementGroup("C3D20TL", m["elements20"], "neohookewa", p),
                                ElementGroup("C3D8TL", m["elements8"], "neohookewa", p)], ties=m["ties"])  # fmt: skip
    dirs = [DirichletBC(m["nodeSets"]["gen_left"], {0: 0.0, 1: 0.0, 2: 0.0}),
            DirichletBC(m["nodeSets"]["gen_right"], {0: -0.3 * 60 * h})]  # fmt: skip
    s = NISTGPU(model, dirs, linsolver=LinSolverOptions(method="fgmres", rtol=1e-8))
    step = Step(maxInc=1.0 / 40, minInc=1e-6, maxIter=25)
    _lib.check(s.lib.ef_set_dirichlet(s.ctx, s.dirIdxHost.ctypes.data, s.dirIdxHost.size), "dir")
    U, dU, P = s._vec(), s._vec(), s._vec()
    prev = None
    stepper = AdaptiveTimeStepper(0.0, 1.0, step.startInc, step.maxInc, step.minInc, step.maxNumInc)
    gen = stepper.generateTimeStep()

    def increment():
        nonlocal U, dU, P, prev
        ts = next(gen)
        s.krylovIterations.clear()
        Unp, dU, P, it = s.solveIncrement(U, dU, P, ts, prev, step)
        _lib.check(s.lib.ef_accept_state(s.ctx), "accept")
        U, prev = Unp, ts
        return it, sum(s.krylovIterations)

    for _ in range(max(3, warmup)):
        increment()
    clocks = ClockSampler()
    clocks.start()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    l0 = s.lib.ef_kernel_launches()
    e0.record()
    its = [increment() for _ in range(steps)]
    e1.record()
    torch.cuda.synchronize()
    launches = s.lib.ef_kernel_launches() - l0
    clk = clocks.stop()
    t = e0.elapsed_time(e1) / 1e3 / steps
    peaks, peak_kind = measured_peaks()
    line = {
        "metric": "tied hex20|hex8 NeoHookeWa box: load-increment s",
        "value": t, "unit": "s", "n_gpus": 1, "steps": steps, "warmup": max(3, warmup), "ms_per_step": t * 1e3,
        "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64 kinematics/stress/residual, f32 stiffness + Krylov inner, f64 refinement",
        "data": "synthetic (structured mesh)",
        "config": {"workload": "60x30x30 box, 27000 C3D20TL (27 Gauss points) | 27000 C3D8TL, NeoHookeWa [80, 200], "
                               "tied interface, 30 % compression in 40 increments", "dofs": int(s.nDof),
                   "ties": int(len(m["ties"][0]))},
        "newton_krylov_per_step": its,
        "solver": f"FGMRES(40) + {multigrid_description()}",
        "gpu_launches": int(launches), "clocks": clk, "peak_kind": peak_kind,
    }  # fmt: skip
    return line


def _element_sample(args):
    """Oracle element pass + CSR update over elements [lo, hi) of the box (one worker)."""
    nx, ny, nz, lo, hi = args
    from oracle.element import SmallStrainElements
    from oracle.mesh import BoxMesh
    from oracle.system import csr_slot_map, csr_update, element_dofs, vij_pattern

    m = BoxMesh(nx, ny, nz, 0.1 * nx, 0.1 * ny, 0.1 * nz)
    els = SmallStrainElements("C3D8", m.coords[m.elements[lo:hi]], "vonmises", PROPS)
    rng = np.random.default_rng(lo)
    dU = rng.normal(0, 2e-4, (hi - lo, 24))
    ed = element_dofs(m.elements[lo:hi])
    I, J = vij_pattern(ed)
    _, indices, x = csr_slot_map(I, J, 3 * m.nNodes)
    t0 = time.perf_counter()
    Ke, _ = els.compute_yourself(dU, dU)
    t1 = time.perf_counter()
    csr_update(Ke.reshape(-1), x, len(indices))
    t2 = time.perf_counter()
    return t1 - t0, t2 - t1, Ke[0].reshape(-1)


def cpu_elastic_system(a):
    """The first Newton system of the box's first loading increment on the CPU: the tangent
    assembled by the oracle's element loop and CSR scatter (every element of the structured box
    has the same geometry, so one element's elastic Ke is scattered into all VIJ slots), the
    clamped face and the pulled face's x DOFs eliminated, the right-hand side the lifted
    prescribed displacement of that increment (u_x = 0.05 * 0.002 lX).  Returns (K_ff, b, D^-1, K)."""
    import scipy.sparse as sp

    from oracle.element import SmallStrainElements
    from oracle.mesh import BoxMesh
    from oracle.system import csr_slot_map, csr_update, element_dofs, vij_pattern

    m = BoxMesh(a.nx, a.ny, a.nz, 0.1 * a.nx, 0.1 * a.ny, 0.1 * a.nz)
    el = SmallStrainElements("C3D8", m.coords[m.elements[:1]], "vonmises", PROPS)
    z = np.zeros((1, 24))
    ke0 = el.compute_yourself(z, z)[0][0].reshape(-1)
    nn = 3 * m.nNodes
    I, J = vij_pattern(element_dofs(m.elements))
    indptr, indices, x = csr_slot_map(I, J, nn)
    del I, J
    data = csr_update(np.tile(ke0, m.nEl), x, len(indices))
    del x
    K = sp.csr_matrix((data, indices, indptr), shape=(nn, nn))
    left, right = m.nodeSets["gen_left"], m.nodeSets["gen_right"]
    dirDofs = np.concatenate([(3 * left[:, None] + np.arange(3)).ravel(), 3 * right])
    u = np.zeros(nn)
    u[3 * right] = 0.05 * 0.002 * 0.1 * a.nx
    free = np.ones(nn, bool)
    free[dirDofs] = False
    b = -(K @ u)[free]
    Kff = K[free][:, free].tocsr()
    return Kff, b, 1.0 / Kff.diagonal(), K


def cpu_jacobi_cg(A, b, dinv, rtol=1e-8, maxIter=None):
    """Scalar Jacobi-preconditioned CG in FP64 (scipy CSR products, one thread) until
    |b - A x| / |b| <= rtol (recurrence residual) or maxIter; returns (iterations, seconds per
    iteration, relative residual)."""
    x = np.zeros_like(b)
    r = b.copy()
    z = dinv * r
    p = z.copy()
    rz = r @ z
    nb = np.sqrt(b @ b)
    it = 0
    t0 = time.perf_counter()
    while np.sqrt(r @ r) > rtol * nb and (maxIter is None or it < maxIter):
        q = A @ p
        al = rz / (p @ q)
        x += al * p
        r -= al * q
        z = dinv * r
        rz2 = r @ z
        p = z + (rz2 / rz) * p
        rz = rz2
        it += 1
    return it, (time.perf_counter() - t0) / max(it, 1), float(np.sqrt(r @ r) / nb)


def cpu_element_sample(a, procs=1, sample=4000, pool=None):
    """The oracle's element loop + CSR update over `sample` elements of the box, split over
    `procs` worker processes (`pool`, a spawned multiprocessing pool, or one spawned here), each
    timed over its own share (the sample's time is the slowest worker's); returns (element-loop s,
    CSR-update s, elements sampled) with the times scaled to the whole box."""
    nEl = a.nx * a.ny * a.nz
    sub = min(nEl, sample)
    chunks = np.linspace(0, sub, procs + 1).astype(int)
    jobs = [(a.nx, a.ny, a.nz, int(chunks[i]), int(chunks[i + 1])) for i in range(procs)]
    if pool is not None:
        res = pool.map(_element_sample, jobs)
    elif procs > 1:
        import multiprocessing as mp

        with mp.get_context("spawn").Pool(procs) as p:
            res = p.map(_element_sample, jobs)
    else:
        res = [_element_sample(jobs[0])]
    return max(r[0] for r in res) * nEl / sub, max(r[1] for r in res) * nEl / sub, sub


def cpu_krylov_measurement(a, system=None):
    """Jacobi-CG to 1e-8 on the CPU on the box's real first Newton system (elastic tangent;
    `system` passes an already assembled one in): the Krylov count per solve and the time per
    iteration, both measured, nothing scaled."""
    t0 = time.time()
    A, b, dinv, _ = cpu_elastic_system(a) if system is None else system
    t_sys = time.time() - t0
    it, t_it, rel = cpu_jacobi_cg(A, b, dinv, rtol=1e-8, maxIter=50000)
    return {"krylov_per_solve": it, "cg_iteration_s": t_it, "relres": rel, "dofs_free": int(b.size),
            "assembly_s": t_sys, "solve_s": it * t_it}  # fmt: skip


def cpu_load_step(newton, t_el, t_csr, krylov_per_solve, t_it):
    """Load-step seconds of the CPU path from measured parts: per Newton iteration one element
    loop, one CSR update and one Jacobi-CG solve of the measured length."""
    return newton * (t_el + t_csr + krylov_per_solve * t_it)


def cpu_baseline(a, newton_per_step, procs=1, sample=4000, krylov=None):
    """CPU baseline of one load step from measured parts: the oracle's element loop + CSR update
    on a bounded element sample (scaled to the whole box by the element count), and a Jacobi-CG
    solve to 1e-8 of the box's real first Newton system run to completion on the CPU (its count
    and time per iteration; `krylov` passes an earlier measurement in).  The load step charges
    `newton_per_step` Newton iterations, each an element pass, a CSR update and one such solve."""
    t_start = time.time()
    t_el, t_csr, sub = cpu_element_sample(a, procs, sample)
    if krylov is None:
        krylov = cpu_krylov_measurement(a)
    nEl = a.nx * a.ny * a.nz
    value = cpu_load_step(newton_per_step, t_el, t_csr, krylov["krylov_per_solve"], krylov["cg_iteration_s"])
    return {
        "value": value,
        "unit": "s",
        "cores": procs,
        "kind": "port",
        "extrapolated": True,
        "sample": f"element loop + CSR update of {sub} of {nEl} elements on {procs} process(es), scaled x{nEl / sub:.0f}; "
                  f"Jacobi-CG (scipy, 1 thread) run to {krylov['relres']:.1e} on the full {krylov['dofs_free']}-DOF "
                  f"first Newton system (elastic tangent): {krylov['krylov_per_solve']} iterations, measured; "
                  f"{newton_per_step} Newton iterations per load step; wall {time.time() - t_start:.0f}s",
        "newton_per_step": newton_per_step,
        "element_loop_s": t_el,
        "csr_update_s": t_csr,
        "element_scale": nEl / sub,
        "krylov_per_solve": krylov["krylov_per_solve"],
        "cg_iteration_s": krylov["cg_iteration_s"],
        "cg_solve_s": krylov["solve_s"],
    }  # fmt: skip


def run_reference(a):
    """The reference's CPU path for the workload, timed through the oracle restatement on the
    host cores (the reference is Python + Cython and does not travel to the GPU machine).

    One step is one bounded sample of the load step: the element loop + CSR update of a share of
    the elements on every host core, and CG_SAMPLE Jacobi-CG iterations on the full system.  The
    Krylov count per solve comes from one Jacobi-CG solve to 1e-8 run to completion before the
    timed steps.  `value` is the load step extrapolated from the steps' parts (flagged
    "extrapolated"); `ms_per_step` is the measured wall time of one sample step."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    t0 = time.time()
    import multiprocessing as mp

    procs = max(1, min(16, os.cpu_count() or 1))
    system = cpu_elastic_system(a)
    A, b, dinv, _ = system
    kry = cpu_krylov_measurement(a, system)
    parts, walls = [], []
    with mp.get_context("spawn").Pool(procs) as pool:
        for _ in range(max(0, a.warmup)):  # untimed, on a small sample (worker start-up, imports, caches)
            cpu_element_sample(a, procs, 250 * procs, pool)
        for _ in range(max(1, a.steps)):
            w0 = time.perf_counter()
            t_el, t_csr, sub = cpu_element_sample(a, procs, 1000 * procs, pool)
            _, t_it, _ = cpu_jacobi_cg(A, b, dinv, rtol=0.0, maxIter=CG_SAMPLE)
            walls.append(time.perf_counter() - w0)
            parts.append((t_el, t_csr, t_it))
    t_el, t_csr, t_it = (float(np.median([p[i] for p in parts])) for i in range(3))
    v = cpu_load_step(PCG_NEWTON_PER_STEP, t_el, t_csr, kry["krylov_per_solve"], t_it)
    ms = 1e3 * float(np.mean(walls))
    nEl = a.nx * a.ny * a.nz
    cb = {
        "value": v, "unit": "s", "cores": procs, "kind": "port", "extrapolated": True,
        "sample": f"per step: element loop + CSR update of {sub} of {nEl} elements on {procs} processes (scaled "
                  f"x{nEl / sub:.0f}) and {CG_SAMPLE} Jacobi-CG iterations on the full {b.size}-DOF system (scipy, 1 "
                  f"thread); Krylov count {kry['krylov_per_solve']} per solve from one Jacobi-CG solve to "
                  f"{kry['relres']:.1e} of the first Newton system, run to completion; {PCG_NEWTON_PER_STEP} Newton "
                  f"iterations per load step",
        "newton_per_step": PCG_NEWTON_PER_STEP, "element_loop_s": t_el, "csr_update_s": t_csr,
        "element_scale": nEl / sub, "krylov_per_solve": kry["krylov_per_solve"], "cg_iteration_s": t_it,
        "cg_solve_measured_s": kry["solve_s"],
    }  # fmt: skip
    line = {
        "impl": "reference",
        "metric": METRIC,
        "value": v,
        "unit": "s",
        "n_gpus": int(os.environ.get("WORLD_SIZE", "1")),
        "steps": len(walls),
        "warmup": max(0, a.warmup),
        "ms_per_step": ms,
        "extrapolated": True,
        "higher_is_better": False,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic (structured box mesh, seeded parameters)",
        "config": workload(a),
        "solver": "element loop + serial CSR scatter + Jacobi-CG (the reference's linSolver slot), CPU",
        "timing": "ms_per_step is the measured wall time of one sample step; value is the load step extrapolated "
                  "from the sampled parts",
        "cpu_baseline": cb,
        "e2e": {"value": v, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "wall_s": time.time() - t0,
    }  # fmt: skip
    print(json.dumps(line), flush=True)


def run_profile(a):
    """Short kernel sequence for ncu: geometry, one element pass, condensation, BSR scatter, block-Jacobi
    setup and one solve capped at 200 (PCG) or 60 (FGMRES) iterations on the full system."""
    import torch

    from edelweissfe_gb300 import _lib
    from edelweissfe_gb300 import build as b
    from edelweissfe_gb300.solver import LinSolverOptions, TimeStep

    b.build()
    learned = a.profile_learned and a.method == "fgmres"
    cap = 5 if learned else (200 if a.method == "pcg" else 60)
    s = build_solver(a, LinSolverOptions(method=a.method, rtol=1e-8, maxIter=cap, maxRefine=1))
    _lib.check(s.lib.ef_set_dirichlet(s.ctx, s.dirIdxHost.ctypes.data, s.dirIdxHost.size), "dir")
    if learned:
        s.initLearnedPreconditioner(seed=0, maxSamples=0)
        p, sc = s.learnedParameters()
        p[-3 * 64:] = np.random.default_rng(0).normal(scale=0.05, size=3 * 64)  # non-zero output layer
        s.setLearnedParameters(p, sc)
        s.enableLearnedPreconditioner(True)
    ts = TimeStep(1, 0.05, 0.05, 0.05, 0.05, 0.05)
    dU = s._vec()
    dU[s.dirIdx] = torch.as_tensor(np.concatenate([d.getDelta(ts) for d in s.dirichlets]), device=dU.device)
    P, F = s._vec(), s._vec()
    s.computeElements(dU, dU, P, F, ts)
    s.assembleStiffnessCSR()
    R = s._vec()
    R[s.dirIdx] = dU[s.dirIdx]
    try:
        s.linearSolve(R)
    except Exception:
        pass
    torch.cuda.synchronize()
    print(json.dumps({"profile": True, "krylov": s.krylovIterations, "nBlocks": s.info.nBlocks}))


if __name__ == "__main__":
    args = parse()
    if args.profile:
        run_profile(args)
    elif args.workload == "cubes" and args.impl == "ours":
        run_cubes(args)
    elif args.workload == "tied" and args.impl == "ours":
        run_tied(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)
