#!/usr/bin/env python
"""Benchmark of the mechanical hot path on one GB300.

Workload: linear-elastic HEX20 block 10 x 4 x 4 m meshed 100 x 40 x 40
(669 161 nodes, 2 007 483 DOFs), 3x3x3 Gauss points, Young's modulus per
element lognormal(ln 30e3, 0.3) from a fixed seed, nu = 0.2, base z=0 fixed,
uniform pressure 1.0 on the top face.  A step is one linear load increment
of the staged Newton solver (mech_stage_solver!): device assembly of K (FP64
element integration + deterministic scatter), FP32 PCG preconditioned by
aggregation multigrid (or block-Jacobi with --solver mixed) inside FP64
iterative refinement to a relative residual of 1e-8, the internal-force
update with the constitutive state and the equilibrium check.  `value` is
DOFs per second of that step with all inputs resident in HBM; `e2e` is the
same step through the C ABI with host buffers (H2D of the stage's essential
values and loads, D2H of displacements and reactions inside the timed region).

--impl reference times the CPU restatement of the reference's own path
(mount_K + sparse direct solve + update_state!) on the host cores, on a
bounded sample of the same workload family.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in (ROOT, os.path.join(ROOT, "amaru.jl_gb300")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402

METRIC = "assembled DOF/s; solve time to 1e-8 rel. residual vs FP64; served p50/p99"
SEED = 0xA11A


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--mesh", default="100x40x40", help="HEX20 divisions nx x ny x nz of the 10x4x4 block")
    ap.add_argument("--cpu-mesh", default="20x8x8", help="bounded CPU sample of the same workload family")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--solver", default="amg", choices=["amg", "mixed"],
                    help="preconditioner of the FP32 PCG in the step: aggregation multigrid or block-Jacobi")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched-models measurement")
    ap.add_argument("--no-serve", action="store_true", help="skip the serving measurement")
    ap.add_argument("--no-recovery", action="store_true", help="skip the nodal recovery measurement")
    ap.add_argument("--no-dyn", action="store_true", help="skip the dynamic (Newmark) stage measurement")
    ap.add_argument("--no-modal", action="store_true", help="skip the modal analysis measurement")
    ap.add_argument("--no-vtu", action="store_true", help="skip the VTU output measurement")
    ap.add_argument("--serve-requests", type=int, default=256)
    ap.add_argument("--slope", default="100x17x40", help="TET10 slope stage divisions (408 000 elements by default)")
    ap.add_argument("--no-slope", action="store_true", help="skip the TET10 slope stage measurement")
    ap.add_argument("--no-coupled", action="store_true", help="skip the hydromechanical mount measurement")
    ap.add_argument("--amg-solve-only", action="store_true",
                    help="profile driver: assemble the --mesh workload, run --steps multigrid solves, print their "
                         "times and exit")
    ap.add_argument("--batch-only", type=int, default=0,
                    help="profile driver: run the batched-models leg alone with this many models and exit")
    return ap.parse_args()


def dims(s):
    return tuple(int(v) for v in s.lower().split("x"))


def rank_info():
    r = int(os.environ.get("RANK", "0"))
    w = int(os.environ.get("WORLD_SIZE", "1"))
    return r, w


def max_over_ranks(vals, device="cpu"):
    """Element-wise maximum of a list of floats over all ranks (a barrier first, so that every rank has
    left its timed region); the values themselves on one process."""
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return [float(v) for v in vals]
    import torch
    dist.barrier()
    t = torch.tensor([float(v) for v in vals], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(v) for v in t.cpu().tolist()]


# ---------------------------------------------------------------------------
# clocks sampled during the timed region
class Clocks:
    def __init__(self):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.p = subprocess.Popen(["nvidia-smi", "--query-gpu=" + q, "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None

    def stop(self):
        if self.p is None:
            return None
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except Exception:
            self.p.kill()
        self.f.flush()
        rows = []
        with open(self.f.name) as fh:
            for ln in fh:
                parts = [x.strip() for x in ln.split(",")]
                if len(parts) >= 9 and parts[1].replace(".", "").isdigit():
                    rows.append(parts)
        os.unlink(self.f.name)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for n, v in zip(names, r[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": float(rows[0][2]), "samples": len(rows),
                "reasons": sorted(reasons), "power_w_max": max(float(r[3]) for r in rows if r[3][0].isdigit())}


# ---------------------------------------------------------------------------
def workload_gpu(nx, ny, nz):
    import amaru_gpu as A
    mesh = A.Mesh(A.Block([[0, 0, 0], [10.0, 4.0, 4.0]], nx=nx, ny=ny, nz=nz, cellshape=A.HEX20))
    ne = len(mesh.shape)
    E = np.exp(np.random.default_rng(SEED).normal(np.log(30e3), 0.3, ne))
    model = A.FEModel(mesh, [("all", A.LinearElastic(E=30e3, nu=0.2))], nips=27, E=E)
    setup = model.configure_dofs([("z==0", A.SurfaceBC(ux=0, uy=0, uz=0)), ("z==4", A.SurfaceBC(tz=-1.0))])
    Uex, Fex = model.get_bc_vals(setup)
    return model, Uex, Fex


def run_ours(a):
    import torch

    import amaru_gpu as A
    from amaru_gpu import _lib as L
    rank, world = rank_info()
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    nx, ny, nz = dims(a.mesh)
    t0 = time.perf_counter()
    model, Uex, Fex = workload_gpu(nx, ny, nz)
    setup_s = time.perf_counter() - t0
    dev = model.dev
    sizes = dev.sizes()
    ndofs = model.ndofs
    step_method = L.SOLVER_AMG if a.solver == "amg" else L.SOLVER_MIXED
    lin = L.default_solve_opts(method=step_method, rtol=1e-8)
    prm = L.default_stage_params(nincs=1, linear=lin)
    d_Uex = torch.from_numpy(Uex).cuda()
    d_Fex = torch.from_numpy(Fex).cuda()
    d_U = torch.zeros(ndofs, dtype=torch.float64, device="cuda")
    d_F = torch.zeros(ndofs, dtype=torch.float64, device="cuda")

    def step():
        rc, st = dev.stage_run_dev(d_Uex.data_ptr(), d_Fex.data_ptr(), prm, d_U.data_ptr(), d_F.data_ptr())
        if rc != 0:
            raise RuntimeError("stage failed: %s" % dev.last_error())
        return st

    for _ in range(a.warmup):
        step()
    torch.cuda.synchronize()
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
    launches0 = dev.launch_count()
    clk = Clocks()
    times, solve_s, kry = [], [], []
    for _ in range(a.steps):
        torch.cuda.synchronize()
        st = step()
        torch.cuda.synchronize()
        times.append(st.seconds)
        solve_s.append(st.solve_seconds)
        kry.append(st.krylov_iterations)
    clocks = clk.stop()
    launches = dev.launch_count() - launches0
    # replicas: every rank solves its own copy of the model; the slowest rank sets the job's time
    mean_step, t_step = max_over_ranks([float(np.mean(times)), max(times)], device="cuda")
    value = world * ndofs / mean_step

    # roofline of the dominant kernel (FP32 BSR SpMV), timed on the library's stream
    spmv_t, spmv_b = dev.time_kernel(L.KERNEL_SPMV32, 50)
    res_t, res_b = dev.time_kernel(L.KERNEL_RESIDUAL64, 10)
    peaks = {}
    pp = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(pp):
        peaks = json.load(open(pp))
    hbm = peaks.get("hbm_gbs")
    peak_kind = "measured" if hbm else "fallback"
    hbm = hbm or 6800.0
    def measured_traffic(name):
        # DRAM bytes per launch from an ncu capture of the kernel, scaled per block and per node
        tp = os.path.join(ROOT, "profiles", name)
        if not os.path.exists(tp):
            return None
        try:
            tj = json.load(open(tp))
            return tj["bytes_per_block"] * sizes["nblocks"] + tj["bytes_per_node"] * sizes["nnodes"]
        except Exception:
            return None

    # the dominant kernel of the step: with the multigrid, the cycle's fine residual r = b - K32 x
    # (four launches per PCG iteration); with block-Jacobi, the PCG's SpMV
    spmv = {"kernel": "k_spmv32v<3> (FP32 BSR SpMV q = K p with fused p.q, padded direction)",
            "bytes_per_launch": spmv_b,
            "avg_launch_s": spmv_t, "achieved": spmv_b / spmv_t / 1e9,
            "traffic": measured_traffic("spmv32v_traffic.json")}
    if step_method == L.SOLVER_AMG:
        amg_t, amg_b = dev.time_kernel(L.KERNEL_AMG_RESIDUAL, 50)
        dom = {"kernel": "k_bsr_res16<3> (multigrid cycle's fine residual r = b - K x from the FP16 copy of the "
                         "scaled matrix)", "bytes_per_launch": amg_b,
               "avg_launch_s": amg_t, "achieved": amg_b / amg_t / 1e9,
               "traffic": measured_traffic("bsr_res16_traffic.json")}
    else:
        dom = spmv
    achieved = dom["achieved"]
    traffic = dom["traffic"]

    # solve-only comparison, same K and RHS: each mixed-precision solver (FP32 PCG in FP64 refinement) against
    # its all-FP64 comparator, the same Krylov method and preconditioner with every operand in FP64
    solve_cmp = {}
    fp64_peak = None
    if not a.no_fp64:
        fp64_peak = fp64_peak_tflops()
        U0 = Uex.copy()
        F0 = Fex.copy()
        runs, kern = {}, {}
        for name, meth in (("amg", L.SOLVER_AMG), ("amg_fp64", L.SOLVER_AMG_FP64), ("mixed", L.SOLVER_MIXED),
                           ("fp64", L.SOLVER_FP64)):
            runs[name] = dev.solve(U0, F0, L.default_solve_opts(method=meth, rtol=1e-8, max_iters=200000))
            if name == "amg_fp64":  # the FP64 cycle's fine residual, on the hierarchy this solve built
                kern["amg_residual64"] = dev.time_kernel(L.KERNEL_AMG_RESIDUAL64, 20)
            if name == "fp64":
                kern["spmv64"] = dev.time_kernel(L.KERNEL_SPMV64, 20)
        # the multigrid solve with the tentative (unsmoothed) prolongators, for the smoothing's share
        dev.set_amg_smoothing(False)
        try:
            runs["amg_unsmoothed"] = dev.solve(U0, F0, L.default_solve_opts(method=L.SOLVER_AMG, rtol=1e-8,
                                                                            max_iters=200000))
        finally:
            dev.set_amg_smoothing(True)
        nu = model.nu
        ref = np.abs(runs["fp64"][0][:nu]).max()
        flops64 = 2.0 * 9 * sizes["nblocks"]  # one FP64 FMA per scalar nonzero
        fp64_kernels = {}
        for kname, (kt, kb) in kern.items():
            fp64_kernels[kname] = {"avg_launch_s": kt, "bytes_per_launch": kb, "achieved_gbs": kb / kt / 1e9,
                                   "hbm_frac": kb / kt / 1e9 / hbm, "fp64_tflops": flops64 / kt / 1e12,
                                   "fp64_frac": flops64 / kt / 1e12 / fp64_peak}
        for name, (U_, F_, st) in runs.items():
            solve_cmp[name + "_s"] = st.seconds
            solve_cmp[name + "_iters"] = st.iterations
            solve_cmp[name + "_rel_residual"] = st.rel_residual
        solve_cmp.update({
            "step_solver": a.solver,
            # the honest ratios: the same method with FP32 Krylov vectors and matrix copy against all-FP64
            "speedup_vs_fp64_same_method": {"multigrid": runs["amg_fp64"][2].seconds / runs["amg"][2].seconds,
                                            "block_jacobi": runs["fp64"][2].seconds / runs["mixed"][2].seconds},
            # the step's solver against the FP64 block-Jacobi PCG (a method and a precision change together)
            "speedup_vs_fp64_block_jacobi": runs["fp64"][2].seconds / runs["amg" if a.solver == "amg"
                                                                            else "mixed"][2].seconds,
            "max_rel_dU_vs_fp64": {n: float(np.abs(runs[n][0][:nu] - runs["fp64"][0][:nu]).max() / ref)
                                   for n in ("amg", "amg_fp64", "mixed", "amg_unsmoothed")},
            "fp64_kernels": fp64_kernels, "fp64_peak_tflops": fp64_peak,
            "fp64_peak_source": "measured: amr_measure_peak (FP64 FMA chains on every SM, CUDA events)"})

    # mount_K at full size: the fast pair-tensor kernel the Newton loop uses, the reference-order kernel whose
    # stored pattern follows the reference's |Ke_ij| >= eps() decisions, and the export in the reference's CSC
    # layout (device conversion, copy to host)
    def wall(f, reps=3):
        ts = []
        for _ in range(reps):
            torch.cuda.synchronize()
            t1 = time.perf_counter()
            f()
            torch.cuda.synchronize()
            ts.append(time.perf_counter() - t1)
        return float(np.median(ts))
    assembly = {"fast_s": wall(dev.assemble_K)}
    dev.set_assembly(L.ASSEMBLY_REFERENCE)
    try:
        assembly["reference_order_s"] = wall(dev.assemble_K)
        t1 = time.perf_counter()
        Kc = dev.K_csc()
        assembly["csc_export_s"] = time.perf_counter() - t1
        assembly["csc_nnz"] = int(Kc.nnz)
        del Kc
    finally:
        dev.set_assembly(L.ASSEMBLY_FAST)
    assembly["fast_dof_per_s"] = ndofs / assembly["fast_s"]
    assembly["reference_order_dof_per_s"] = ndofs / assembly["reference_order_s"]
    dev.assemble_K()  # K current again (the timing below reads it, and leaves it as it is)
    st_t, st_fl = dev.time_kernel(L.KERNEL_STIFFNESS, 5)
    pk64 = fp64_peak_tflops()
    # the operation count is that of the pair form in FP64; in 3-D the pair sums (3/4 of it) and the blocks run in
    # float-float on the FP32 pipe, so the rate is an FP64-equivalent rate and may exceed the FP64 FMA peak
    assembly["stiffness_kernel"] = {"kernel": "stiffness_kernel<3, 20> (pair-tensor element stiffness: FP64 geometry, "
                                              "float-float pair sums and blocks)",
                                    "avg_launch_s": st_t, "elements_per_s": sizes["nelems"] / st_t,
                                    "fp64_equivalent_flops_per_launch": st_fl,
                                    "fp64_equivalent_tflops": st_fl / st_t / 1e12, "fp64_peak_tflops": pk64}

    # e2e: the same step through the C ABI with host buffers (H2D inputs, D2H results inside), the buffers in
    # pinned host memory
    def pinned(v):
        return torch.from_numpy(np.ascontiguousarray(v, dtype=np.float64)).pin_memory().numpy()
    Uh, Fh = pinned(Uex), pinned(Fex)
    outs = (pinned(np.zeros(ndofs)), pinned(np.zeros(ndofs)))
    rc, _, _, _ = dev.stage_run(Uh, Fh, prm, out=outs)  # untimed: rebuilds what the comparisons above replaced
    if rc != 0:
        raise RuntimeError(dev.last_error())
    e2e_t = []
    for _ in range(a.steps):
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        rc, U, F, st = dev.stage_run(Uh, Fh, prm, out=outs)
        torch.cuda.synchronize()
        e2e_t.append(time.perf_counter() - t1)
        if rc != 0:
            raise RuntimeError(dev.last_error())
    e2e_v = world * ndofs / max_over_ranks([float(np.mean(e2e_t))], device="cuda")[0]

    out = {
        "metric": METRIC, "value": value, "unit": "DOF/s", "n_gpus": world, "steps": a.steps, "warmup": a.warmup,
        "ms_per_step": mean_step * 1e3, "ms_per_step_max": t_step * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": "f64 assembly/residual/state (3-D stiffness pair sums float-float), f32 Krylov", "data": "synthetic",
        "config": {"workload": "HEX20 %dx%dx%d block 10x4x4 m, 27 IP, lognormal E (seed 0xA11A), nu=0.2, base fixed, "
                               "top pressure 1.0; one linear increment: assemble K + PCG(f32, %s)/IR(f64) to 1e-8 + "
                               "internal forces" % (nx, ny, nz, "multigrid" if a.solver == "amg" else "block-Jacobi"),
                   "ndofs": ndofs, "nu": model.nu, "nnodes": sizes["nnodes"], "nelems": sizes["nelems"],
                   "nnz_blocks": sizes["nblocks"], "nnz": sizes["nblocks"] * 9,
                   "l2": "inputs larger than L2 (K32 %.2f GB, K64 %.2f GB)" % (sizes["nblocks"] * 36 / 1e9,
                                                                             sizes["nblocks"] * 72 / 1e9),
                   "parallelism": "replicas (one model per GPU)", "setup_s": setup_s},
        "solve": dict(solve_cmp, step_solve_s=float(np.mean(solve_s)), step_krylov_iters=int(np.mean(kry))),
        "assembly": assembly,
        "roofline": {"bound": "hbm", "kernel": dom["kernel"],
                     "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                     "peak_source": peak_kind, "traffic": traffic, "bytes_per_launch": dom["bytes_per_launch"],
                     "avg_launch_s": dom["avg_launch_s"],
                     "spmv32": dict(spmv, frac=spmv["achieved"] / hbm),
                     "residual64": {"achieved": res_b / res_t / 1e9, "frac": res_b / res_t / 1e9 / hbm,
                                    "avg_launch_s": res_t}},
        "e2e": {"value": e2e_v, "unit": "DOF/s", "h2d_bytes_per_step": 2 * ndofs * 8, "d2h_bytes_per_step": 2 * ndofs * 8,
                "ms_per_step": float(np.mean(e2e_t)) * 1e3},
        "gpu_launches": launches,
        "clocks": clocks,
    }
    # the secondary legs: a failure in one is recorded on the line and does not take the headline with it
    cpu_here = rank == 0 and world == 1 and not a.no_cpu  # the CPU samples: rank 0 of a 1-GPU run
    legs = [("recovery", not a.no_recovery, lambda: recovery_leg(model, cpu_here)),
            ("vtu", not a.no_vtu, lambda: vtu_leg(model, cpu_here)),
            ("dynamic", not a.no_dyn, lambda: dyn_leg(model, cpu_here)),
            ("modal", not a.no_modal, lambda: modal_leg(model, cpu_here)),
            ("batch", not a.no_batch, batch_leg),
            ("serving", not a.no_serve, lambda: serving_leg(a.serve_requests)),
            ("slope", bool(a.slope) and not a.no_slope, lambda: slope_leg(a.slope)),
            ("coupled", not a.no_coupled, lambda: coupled_leg(cpu_here))]
    for name, on, fn in legs:
        if not on:
            continue
        try:
            out[name] = fn()
        except Exception as e:  # noqa: BLE001
            out[name] = {"error": "%s: %s" % (type(e).__name__, e)}
    if cpu_here:
        out["cpu_baseline"] = cpu_baseline(a, steps=1, warmup=0)
    return out


# ---------------------------------------------------------------------------
# Nodal output recovery (nodal_patch_recovery) of the step's IP states on the same
# model: the whole device recovery (IP fields, patch fits, averaging), the same
# call with the result copied to the host, and the patch-fit kernel against the
# FP64 pipe.  The CPU baseline runs the oracle's restatement on a HEX20 8x4x4
# block of the same family with seeded states.
# ---------------------------------------------------------------------------
_PEAKS = {}


def fp64_peak_tflops():
    """FP64 FMA throughput of this GPU, measured once per run (amr_measure_peak)."""
    if "fp64" not in _PEAKS:
        from amaru_gpu import _lib as L
        _PEAKS["fp64"] = L.measure_peak(L.PEAK_FP64_FMA)
    return _PEAKS["fp64"]


def recovery_leg(model, with_cpu, reps=5):
    import torch
    dev = model.dev
    t0 = time.perf_counter()
    names = dev.recovery_fields()
    setup_s = time.perf_counter() - t0
    nn = dev.sizes()["nnodes"]
    d_V = torch.zeros(len(names) * nn, dtype=torch.float64, device="cuda")
    dev.recover_nodal_dev(d_V.data_ptr())  # warm
    ts = []
    for _ in range(reps):
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        dev.recover_nodal_dev(d_V.data_ptr())
        ts.append(time.perf_counter() - t1)
    te = []
    for _ in range(reps):
        t1 = time.perf_counter()
        V, _ = dev.recover_nodal()
        te.append(time.perf_counter() - t1)
    fit_t, flops, nsvd = dev.time_recovery(10)
    out = {"fields": len(names), "nnodes": nn, "structure_setup_s": setup_s,
           "device_s": float(np.mean(ts)), "value": nn / float(np.mean(ts)), "unit": "nodes/s",
           "e2e": {"value": nn / float(np.mean(te)), "unit": "nodes/s", "s": float(np.mean(te)),
                   "d2h_bytes": int(V.size * 8)},
           "patch_fit": {"kernel": "k_patch_fit<3> (warp per patch: Gram/Cholesky fit, moments, nodal values)",
                         "avg_launch_s": fit_t, "flops_per_launch": flops,
                         "achieved": flops / fit_t / 1e12, "unit": "TFLOP/s (FP64)",
                         "peak": fp64_peak_tflops(), "peak_source": "measured FP64 FMA peak (amr_measure_peak)",
                         "frac": flops / fit_t / 1e12 / fp64_peak_tflops(), "svd_patches": nsvd}}
    if with_cpu:
        out["cpu_baseline"] = recovery_cpu_sample()
    return out


def recovery_cpu_sample(n=(8, 4, 4)):
    sys.path.insert(0, ROOT)
    import oracle as O
    mo = O.Mesh(O.Block([[0, 0, 0], [10.0 * n[0] / 100, 4.0 * n[1] / 40, 4.0 * n[2] / 40]], nx=n[0], ny=n[1],
                        nz=n[2], cellshape=O.HEX20))
    om = O.FEModel(mo, [("all", O.LinearElastic(E=30e3, nu=0.2))], nips=27)
    om.state[:, :12] = np.random.default_rng(SEED).normal(size=(len(om.state), 12))
    t0 = time.perf_counter()
    O.nodal_patch_recovery(om)
    dt = time.perf_counter() - t0
    return {"value": om.nnodes / dt, "unit": "nodes/s", "cores": 1, "kind": "port",
            "sample": "oracle nodal_patch_recovery (Python/numpy restatement) on HEX20 %dx%dx%d, 27 IP, %d nodes: "
                      "%.2f s" % (n[0], n[1], n[2], om.nnodes, dt)}


# ---------------------------------------------------------------------------
# VTU output (save(model, "file.vtu")) of the step's model: update_output_data! (dof values and the 16
# recovered fields on the device) and the ascii file, to a scratch file removed afterwards; the writer's
# host threads all, then one.  The CPU baseline is the oracle's Python writer on HEX20 8x4x4.
# ---------------------------------------------------------------------------
def vtu_leg(model, with_cpu):
    d = tempfile.mkdtemp()
    path = os.path.join(d, "out.vtu")
    try:
        t0 = time.perf_counter()
        node, elem = model.update_output_data()
        t_data = time.perf_counter() - t0
        items = (list(node.items()), list(elem.items()))
        res = {}
        for nt in (0, 1):
            t0 = time.perf_counter()
            model.dev.write_vtu(path, *items, nthreads=nt)
            res[nt] = time.perf_counter() - t0
        size = os.path.getsize(path)
    finally:
        if os.path.exists(path):
            os.remove(path)
        os.rmdir(d)
    out = {"bytes": size, "output_data_s": t_data, "write_s": res[0], "write_1thread_s": res[1],
           "threads": os.cpu_count(), "value": size / res[0] / 1e6, "unit": "MB/s",
           "value_1thread": size / res[1] / 1e6}
    if with_cpu:
        out["cpu_baseline"] = vtu_cpu_sample()
    return out


def vtu_cpu_sample(n=(8, 4, 4)):
    sys.path.insert(0, ROOT)
    import oracle as O
    mo = O.Mesh(O.Block([[0, 0, 0], [0.8, 0.4, 0.4]], nx=n[0], ny=n[1], nz=n[2], cellshape=O.HEX20))
    rng = np.random.default_rng(SEED)
    nn = len(mo.coords)
    node = [("node-id", np.arange(1, nn + 1))] + [("f%d" % i, rng.normal(size=nn)) for i in range(22)] + \
           [("U", rng.normal(size=(nn, 3)))]
    ne = len(mo.elems)
    shapes = np.array([c.shape for c in mo.elems])
    conn_ptr = np.concatenate([[0], np.cumsum([len(c.nodes) for c in mo.elems])])
    conn = np.array([v for c in mo.elems for v in c.nodes])
    t0 = time.perf_counter()
    txt = O.vtu.save_vtu(mo.coords, conn_ptr, conn, shapes, node, [("elem-id", np.arange(1, ne + 1))])
    dt = time.perf_counter() - t0
    return {"value": len(txt) / dt / 1e6, "unit": "MB/s", "cores": 1, "kind": "port",
            "sample": "oracle save_vtu (Python) of HEX20 %dx%dx%d with 22 fields + U: %d bytes in %.2f s"
                      % (n[0], n[1], n[2], len(txt), dt)}


# ---------------------------------------------------------------------------
# Dynamic stage (dyn_stage_solver!) on the bench model: density 2.4e-3, base fixed, the top pressure
# applied suddenly, Rayleigh damping alpha = 0.5, beta = 1e-4, tspan 0.01 in 5 increments, the
# multigrid-preconditioned solve to 1e-8.  value = DOFs x increments per second of device time; e2e the
# same through the host-buffer call.  The CPU baseline runs the oracle's restatement on a HEX20 6x3x3
# block of the same family.
# ---------------------------------------------------------------------------
DYN = dict(rho=2.4e-3, alpha=0.5, beta=1e-4, tspan=0.01, nincs=5)


def dyn_leg(model, with_cpu):
    import amaru_gpu as A
    from amaru_gpu import _lib as L
    model.rho[:] = DYN["rho"]
    bcs = [("z==0", A.SurfaceBC(ux=0, uy=0, uz=0)), ("z==4", A.SurfaceBC(tz=-1.0))]
    runs = []
    for _ in range(2):  # the first run includes the multigrid set-up of the new pseudo-stiffness
        ana = A.DynAnalysis(model)
        ana.addstage(bcs, tspan=DYN["tspan"], nincs=DYN["nincs"])
        t0 = time.perf_counter()
        ok, msg = ana.solve(solver="amg", linear_rtol=1e-8, alpha=DYN["alpha"], beta=DYN["beta"])
        wall = time.perf_counter() - t0
        if not ok:
            raise RuntimeError("dynamic stage failed: " + msg)
        runs.append((ana.stats, wall))
    st, wall = runs[-1]
    nd = model.ndofs
    rhs_t, rhs_b = model.dev.time_kernel(L.KERNEL_DYN_RHS, 20)
    out = {"workload": "bench HEX20 model, rho %g, Rayleigh (%g, %g), tspan %g in %d increments, multigrid PCG "
                       "to 1e-8" % (DYN["rho"], DYN["alpha"], DYN["beta"], DYN["tspan"], DYN["nincs"]),
           "ndofs": nd, "increments": st.increments, "newton_iterations": st.iterations,
           "krylov_iterations": st.krylov_iterations, "device_s": st.seconds, "solve_s": st.solve_seconds,
           "value": nd * st.increments / st.seconds, "unit": "DOF-increments/s",
           "e2e": {"value": nd * st.increments / wall, "unit": "DOF-increments/s", "s": wall,
                   "h2d_bytes": 4 * nd * 8, "d2h_bytes": 4 * nd * 8},
           "rhs_kernel": {"kernel": "k_dyn_rhs<3> (base + M x + (alpha M + beta K) y)", "avg_launch_s": rhs_t,
                          "bytes_per_launch": rhs_b, "achieved_gbs": rhs_b / rhs_t / 1e9}}
    # FP64 work per launch: per block 2 B FMA on M (x and y) and B^2 on K; the FP64 pipe bounds it on GB300
    fl = 2.0 * model.dev.sizes()["nblocks"] * (2 * 3 + 9)
    pk = fp64_peak_tflops()
    out["rhs_kernel"].update({"fp64_tflops": fl / rhs_t / 1e12, "fp64_peak_tflops": pk,
                              "fp64_frac": fl / rhs_t / 1e12 / pk})
    if with_cpu:
        out["cpu_baseline"] = dyn_cpu_sample()
    return out


def dyn_cpu_sample(n=(6, 3, 3)):
    sys.path.insert(0, ROOT)
    import oracle as O
    mo = O.Mesh(O.Block([[0, 0, 0], [10.0 * n[0] / 100, 4.0 * n[1] / 40, 4.0 * n[2] / 40]], nx=n[0], ny=n[1],
                        nz=n[2], cellshape=O.HEX20))
    om = O.FEModel(mo, [("all", O.LinearElastic(E=30e3, nu=0.2, rho=DYN["rho"]))], nips=27)
    top = 4.0 * n[2] / 40
    ana = O.DynAnalysis(om)
    ana.addstage([("z==0", O.SurfaceBC(ux=0, uy=0, uz=0)), ("z==%r" % top, O.SurfaceBC(tz=-1.0))],
                 tspan=DYN["tspan"], nincs=DYN["nincs"])
    t0 = time.perf_counter()
    ok, _ = ana.solve(alpha=DYN["alpha"], beta=DYN["beta"])
    dt = time.perf_counter() - t0
    return {"value": ana.ndofs * ana.increments / dt, "unit": "DOF-increments/s", "cores": 1, "kind": "port",
            "sample": "oracle dyn_stage_solver! (C element kernels, Python mount_M, SuperLU) on HEX20 %dx%dx%d, "
                      "%d DOFs, %d increments: %.2f s" % (n[0], n[1], n[2], ana.ndofs, ana.increments, dt)}


# ---------------------------------------------------------------------------
# Modal analysis (mech_modal_solver!) of the bench model, base fixed, density 2.4e-3: the 5 lowest
# modes to a relative residual of 1e-8.  value = unknown DOFs per second of device time.  The CPU
# baseline runs the oracle's restatement (scipy eigsh with SuperLU) on a HEX20 6x3x3 block.
# ---------------------------------------------------------------------------
def modal_leg(model, with_cpu, nmodes=5):
    import amaru_gpu as A
    model.rho[:] = DYN["rho"]
    ana = A.ModalAnalysis(model)
    ana.addstage([("z==0", A.SurfaceBC(ux=0, uy=0, uz=0))])
    t0 = time.perf_counter()
    ana.solve(nmodes=nmodes, tol=1e-8)
    wall = time.perf_counter() - t0
    st = ana.stats
    out = {"workload": "bench HEX20 model, base fixed, rho %g, %d lowest modes, LOBPCG (block %d) with the "
                       "multigrid preconditioner to 1e-8" % (DYN["rho"], nmodes, st.block),
           "nu": model.nu, "omega": [float(w) for w in ana.freqs], "iterations": st.iterations,
           "max_residual": st.max_residual, "device_s": st.seconds, "value": model.nu / st.seconds,
           "unit": "DOF/s", "e2e": {"value": model.nu / wall, "unit": "DOF/s", "s": wall,
                                   "d2h_bytes": int(model.nu * nmodes * 8)}}
    if with_cpu:
        out["cpu_baseline"] = modal_cpu_sample(nmodes)
    return out


def modal_cpu_sample(nmodes, n=(6, 3, 3)):
    sys.path.insert(0, ROOT)
    import oracle as O
    mo = O.Mesh(O.Block([[0, 0, 0], [10.0 * n[0] / 100, 4.0 * n[1] / 40, 4.0 * n[2] / 40]], nx=n[0], ny=n[1],
                        nz=n[2], cellshape=O.HEX20))
    om = O.FEModel(mo, [("all", O.LinearElastic(E=30e3, nu=0.2, rho=DYN["rho"]))], nips=27)
    t0 = time.perf_counter()
    _, _, nu = O.modal(om, [("z==0", O.SurfaceBC(ux=0, uy=0, uz=0))], nmodes)
    dt = time.perf_counter() - t0
    return {"value": nu / dt, "unit": "DOF/s", "cores": 1, "kind": "port",
            "sample": "oracle mech_modal_solver! (C mount_K, Python mount_M, scipy eigsh + SuperLU) on HEX20 "
                      "%dx%dx%d, %d unknown DOFs, %d modes: %.2f s" % (n[0], n[1], n[2], nu, nmodes, dt)}


# ---------------------------------------------------------------------------
# ---------------------------------------------------------------------------
# Batched independent models: 512 plane-strain QUAD8 rectangles 2 x 1, n x n with
# n uniform in [10, 60], E lognormal(ln 200e3, 0.2), nu uniform [0.2, 0.35], 3x3
# Gauss points, left edge fixed, unit traction tx on the right edge; one linear
# stage of all of them through the batched stage driver.
# ---------------------------------------------------------------------------
BATCH_SEED = 0xC4


def _quad8_models(inst, cache, device):
    import amaru_gpu as A
    out = []
    for n, E, nu in inst:
        if n not in cache:
            cache[n] = A.Mesh(A.Block([[0, 0], [2.0, 1.0]], nx=n, ny=n, cellshape=A.QUAD8))
        out.append(A.FEModel(cache[n], [("all", A.LinearElastic(E=E, nu=nu))],
                             A.MechContext(stressmodel="planestrain"), nips=9, device=device))
    return out


def batch_leg(count=512, steps=3):
    """The batched stage of config 4 with the per-part multigrid-preconditioned PCG (the joined model's V-cycle)
    and, beside it, with the per-part block-Jacobi PCG of one persistent launch."""
    import torch
    import amaru_gpu as A
    from amaru_gpu import _lib as L
    rng = np.random.default_rng(BATCH_SEED)
    ns = rng.integers(10, 61, count)
    Es = np.exp(rng.normal(np.log(200e3), 0.2, count))
    nus = rng.uniform(0.2, 0.35, count)
    inst = [(int(a), float(b), float(c)) for a, b, c in zip(ns, Es, nus)]
    bcs = [("x==0", A.SurfaceBC(ux=0, uy=0)), ("x==2", A.SurfaceBC(tx=1.0))]
    cache = {}
    t0 = time.perf_counter()
    ba = A.BatchAnalysis(_quad8_models(inst, cache, False))
    ba.addstage(bcs)
    setup_s = time.perf_counter() - t0
    tu = ba.autotune()
    J = ba.joined
    Uex, Fex = ba.configure(ba.stages[0].bcs)
    dU, dF = torch.from_numpy(Uex).cuda(), torch.from_numpy(Fex).cuda()
    oU, oF = torch.zeros_like(dU), torch.zeros_like(dF)

    def run(method):
        p = L.default_stage_params(linear=L.default_solve_opts(method=method, rtol=1e-8))
        secs, solve, launches = [], [], []
        for r in range(steps + 1):
            c0 = J.dev.launch_count()
            rc, st = J.dev.stage_run_dev(dU.data_ptr(), dF.data_ptr(), p, oU.data_ptr(), oF.data_ptr())
            if rc != 0:
                raise RuntimeError(J.dev.last_error())
            if r > 0:  # the first run is the warm-up
                secs.append(st.seconds)
                solve.append(st.solve_seconds)
                launches.append(J.dev.launch_count() - c0)
        ps = J.dev.part_stats()
        kr = np.array([s.krylov_iterations for s in ps])
        t = float(np.mean(secs))
        out = {"ms_per_batch": t * 1e3, "solve_ms": float(np.mean(solve)) * 1e3, "models_per_s": count / t,
               "dof_per_s": J.ndofs / t, "launches_per_batch": int(np.mean(launches)),
               "krylov_iters_max": int(kr.max()), "krylov_iters_mean": float(kr.mean()),
               "parts_converged": int(sum(s.status == 0 for s in ps))}
        # the same 32 models (every 16th) one at a time on their own handles, against the same 32 batched
        samp = inst[::max(1, count // 32)][:32]
        seq = 0.0
        for m in _quad8_models(samp, cache, True):
            setup = m.configure_dofs(bcs)
            U0, F0 = m.get_bc_vals(setup)
            m.dev.stage_run(U0, F0, p)
            rc, _, _, s1 = m.dev.stage_run(U0, F0, p)
            seq += s1.seconds
            m.dev.close()
        bs = A.BatchAnalysis(_quad8_models(samp, cache, False))
        bs.addstage(bcs)
        Us, Fs = bs.configure(bs.stages[0].bcs)
        bs.joined.dev.stage_run(Us, Fs, p)
        rc, _, _, s2 = bs.joined.dev.stage_run(Us, Fs, p)
        out["sample_32"] = {"one_at_a_time_s": seq, "batched_s": s2.seconds, "speedup": seq / s2.seconds}
        return out

    mg = run(L.SOLVER_AMG)
    bj = run(L.SOLVER_MIXED)
    out = {"workload": "%d plane-strain QUAD8 models 2x1, n x n with n~U{10..60} (seed 0xC4), E lognormal(ln 200e3, "
                       "0.2), nu~U[0.2,0.35], 9 IP, left edge fixed, unit tx on the right edge; one linear stage of "
                       "every model in one batched stage (per-part PCG to 1e-8 preconditioned by the joined model's "
                       "multigrid V-cycle; block_jacobi: per-part block-Jacobi PCG in one persistent launch)" % count,
           "models": count, "ndofs": int(J.ndofs), "solver": "multigrid", "setup_s": setup_s}
    out.update(mg)
    out["block_jacobi"] = bj
    out["tuning"] = {"stiffness_epb": tu.stiffness_epb[0], "internal_epb": tu.internal_epb[0],
                     "pcg_threads": tu.batch_threads, "pcg_ctas_per_sm": tu.batch_ctas_per_sm}
    return out


# ---------------------------------------------------------------------------
# Serving: Poisson arrivals (200 requests/s, seeded) of linear-elastic HEX8
# cantilever blocks 1 x 0.5 x 0.5 with DOFs log-uniform in [1e3, 2e6] and 1..10 increments,
# and at 20 % elastoplastic TET10 blocks (von Mises, gravity + top surcharge,
# automatic increments, DOFs log-uniform in [1e3, 2e5]); continuous batching
# with admission against the free HBM.
# ---------------------------------------------------------------------------
SERVE_SEED = 0xC5


def _serve_requests(count):
    import amaru_gpu as A
    rng = np.random.default_rng(SERVE_SEED)
    arrivals = np.cumsum(rng.exponential(1 / 200.0, count))
    is_tet = np.zeros(count, dtype=bool)
    is_tet[:int(round(0.2 * count))] = True  # exactly 20 % elastoplastic TET10 requests, in seeded order
    rng.shuffle(is_tet)
    reqs = []
    for i in range(count):
        tet = bool(is_tet[i])
        incs = int(rng.integers(1, 11))
        if tet:
            dofs = float(np.exp(rng.uniform(np.log(1e3), np.log(2e5))))
            k = max(1, int(round(((dofs / 3) / 16) ** (1 / 3))))  # nodes ~ (4k+1)(2k+1)^2
            mesh = A.Mesh(A.Block([[0, 0, 0], [1.0, 0.5, 0.5]], nx=2 * k, ny=k, nz=k, cellshape=A.TET10))
            m = A.FEModel(mesh, [("all", A.VonMises(E=50e3, nu=0.3, fy=100.0, H=1e3))], device=False)
            bcs = [("z==0", A.SurfaceBC(ux=0, uy=0, uz=0)), ("z==0.5", A.SurfaceBC(tz=-120.0)),
                   ("all", A.BodyC(wz=-20.0))]
            kw = dict(nincs=incs, autoinc=True, solver="amg")
        else:
            dofs = float(np.exp(rng.uniform(np.log(1e3), np.log(2e6))))
            k = max(1, int(round(((dofs / 3) / 2) ** (1 / 3))))  # nodes ~ (2k+1)(k+1)^2
            mesh = A.Mesh(A.Block([[0, 0, 0], [1.0, 0.5, 0.5]], nx=2 * k, ny=k, nz=k, cellshape=A.HEX8))
            m = A.FEModel(mesh, [("all", A.LinearElastic(E=200e3, nu=0.3))], device=False)
            bcs = [("x==0", A.SurfaceBC(ux=0, uy=0, uz=0)), ("x==1", A.SurfaceBC(tz=-1.0))]
            kw = dict(nincs=incs, solver="amg")
        reqs.append((arrivals[i], "tet10" if tet else "hex8", m, bcs, kw))
    return reqs


def serving_leg(count=32, max_active=8):
    import torch
    from amaru_gpu import serve
    reqs = _serve_requests(count)
    free, _ = torch.cuda.mem_get_info()
    budget = 0.85 * free
    lat, out, failures = [], [], []
    with serve.Server(hbm_budget_bytes=budget, max_active=max_active) as srv:
        t0 = time.perf_counter()
        tickets = []
        for at, kind, m, bcs, kw in reqs:
            wait = at - (time.perf_counter() - t0)
            if wait > 0:
                time.sleep(wait)
            tickets.append(srv.submit(m, bcs, **kw))
        for (at, kind, m, bcs, kw), tk in zip(reqs, tickets):
            rc, U, F, res, msg = srv.wait(tk)
            out.append((kind, rc, res, tk.ndofs))
            if rc != 0:
                failures.append("%s %d DOFs: %s" % (kind, tk.ndofs, msg))
        info = srv.info()
    lat = np.array([r.t_done - r.t_submit for _, _, r, _ in out])
    t_first = min(r.t_submit for _, _, r, _ in out)
    t_last = max(r.t_done for _, _, r, _ in out)
    span = t_last - t_first
    dof_incs = sum(n * r.stage.increments for _, rc, r, n in out if rc == 0)

    def pct(v):
        v = np.asarray(v)
        return {"p50_ms": float(np.percentile(v, 50)) * 1e3, "p99_ms": float(np.percentile(v, 99)) * 1e3}
    # device concurrency: the time-weighted number of requests whose stage is on the GPU (device clock)
    ev = sorted([(r.dev_start, 1) for _, _, r, _ in out] + [(r.dev_end, -1) for _, _, r, _ in out])
    busy, weighted, cur, t_prev = 0.0, 0.0, 0, ev[0][0]
    for t, d in ev:
        if cur > 0:
            busy += t - t_prev
            weighted += cur * (t - t_prev)
        cur += d
        t_prev = t
    return {"workload": "%d requests, Poisson arrivals 200/s (seed 0xC5): HEX8 cantilever blocks 1x0.5x0.5, DOFs log-uniform "
                        "[1e3, 2e6], 1..10 linear increments; exactly 20%% TET10 von Mises blocks (gravity + surcharge, "
                        "automatic increments), DOFs log-uniform [1e3, 2e5]; multigrid-preconditioned solver to 1e-8" % count,
            "requests": count, "completed": int(sum(rc == 0 for _, rc, _, _ in out)),
            "tet10": int(sum(k == "tet10" for k, _, _, _ in out)),
            "solves_per_s": count / span, "p50_ms": float(np.percentile(lat, 50)) * 1e3,
            "p99_ms": float(np.percentile(lat, 99)) * 1e3, "mean_ms": float(lat.mean()) * 1e3,
            "latency_parts": {"queue": pct([r.t_admit - r.t_submit for _, _, r, _ in out]),
                              "host_setup": pct([r.t_stage - r.t_admit for _, _, r, _ in out]),
                              "stage_device": pct([r.stage.seconds for _, _, r, _ in out]),
                              "stage_wall": pct([r.t_done - r.t_stage for _, _, r, _ in out])},
            "device_overlap": {"busy_s": busy, "mean_requests_on_device": weighted / busy if busy else 0.0,
                               "stage_device_s_sum": float(sum(r.stage.seconds for _, _, r, _ in out))},
            "dof_increments_per_s": dof_incs / span, "makespan_s": span, "max_active": max_active,
            "peak_active": int(info.peak_active), "peak_admitted_gb": info.peak_bytes / 1e9,
            "hbm_budget_gb": budget / 1e9,
            "total_dofs": int(sum(n for _, _, _, n in out)), "failures": failures}


# ---------------------------------------------------------------------------
# Nonlinear geomechanics: plane-strain slope extruded along y, TET10 block mesh
# with jittered interior vertices (seed 0xC3), von Mises E=50e3 nu=0.3 fy=100
# H=1e3, gravity 20 + crest surcharge 200 ramped over 20 increments, Newton tol 1e-6.
# ---------------------------------------------------------------------------
def slope_leg(spec):
    import amaru_gpu as A
    from amaru_gpu import workloads as W
    n = dims(spec)
    g = W.SLOPE
    t0 = time.perf_counter()
    mesh = A.Mesh(A.Block([[0, 0, 0], [g["L"], g["W"], g["H"]]], nx=n[0], ny=n[1], nz=n[2], cellshape=A.TET10))
    mesh.coords = W.slope_coords(mesh.coords, mesh.elem_nodes(), W.boundary_nodes(mesh), 4, *n, seed=0xC3)
    model = A.FEModel(mesh, [("all", A.VonMises(E=50e3, nu=0.3, fy=100.0, H=1e3))])
    ana = A.MechAnalysis(model)
    ana.addstage(W.slope_bcs(A, 200.0), nincs=20)
    setup_s = time.perf_counter() - t0
    ok, msg = ana.solve(tol=1e-6, solver="amg")
    st = ana.stats[0]
    sizes = model.dev.sizes()
    plastic = int((model.state()[:, 12] > 0).sum())
    return {"workload": "TET10 slope %s (L=10, W=1.7, crest 4 m, toe 2 m, jittered interior, seed 0xC3), von Mises "
                        "E=50e3 nu=0.3 fy=100 H=1e3, gravity 20 + crest surcharge 200 over 20 increments, Newton "
                        "tol 1e-6, multigrid-preconditioned solver to 1e-8" % spec,
            "ok": bool(ok), "message": msg, "ndofs": int(model.ndofs), "nelems": sizes["nelems"],
            "nnodes": sizes["nnodes"], "increments": st.increments, "newton_iterations": st.iterations,
            "krylov_iterations": st.krylov_iterations, "stage_s": st.seconds, "solve_s": st.solve_seconds,
            "dof_iterations_per_s": model.ndofs * st.iterations / st.seconds, "plastic_ips": plastic,
            "setup_s": setup_s}


# ---------------------------------------------------------------------------
# Hydromechanical mount (hm_mount_global_matrices): HEX20 block 3 x 1.2 x 1.2 meshed 30 x 12 x 12, linear
# elastic skeleton (E 1e4, nu 0.25), Biot alpha 0.9, permeability 2.5e-3, storativity 1e-4, gammaw 10, dt 0.05;
# base fixed, top drained.  value = DOFs per second of the whole call (device mount, CSC export to the host).
# The CPU baseline runs the oracle's restatement on HEX20 3 x 2 x 2.
# ---------------------------------------------------------------------------
def _coupled_case(M, CPm, n):
    box = [[0, 0, 0], [0.1 * n[0], 0.1 * n[1], 0.1 * n[2]]]
    mesh = M.Mesh(M.Block(box, nx=n[0], ny=n[1], nz=n[2], cellshape=M.HEX20))
    model = M.FEModel(mesh, [("all", M.LinearElastic(E=1e4, nu=0.25))])
    z = np.asarray(mesh.coords)[:, 2]
    pres = np.zeros((len(z), 4), dtype=bool)
    pres[np.isclose(z, 0.0), :3] = True
    pres[np.isclose(z, z.max()), 3] = True
    eq4, nd, nu = CPm.coupled_dofs(model, pres)
    prm = np.tile([0.9, 2.5e-3, 1e-4], (len(model.shape) if hasattr(model, "shape") else len(mesh.shape), 1))
    return model, eq4, nd, prm


def coupled_leg(with_cpu, n=(30, 12, 12), reps=3):
    import amaru_gpu as A
    from amaru_gpu import coupled as CP
    model, eq4, nd, prm = _coupled_case(A, CP, n)
    phi = np.zeros(nd)
    G, _ = CP.mount_coupled(model, CP.HYDRO, prm, eq4, nd, 0.05, phi, gammaw=10.0)  # warm
    ts = []
    for _ in range(reps):
        t0 = time.perf_counter()
        G, R = CP.mount_coupled(model, CP.HYDRO, prm, eq4, nd, 0.05, phi, gammaw=10.0)
        ts.append(time.perf_counter() - t0)
    t = float(np.median(ts))
    out = {"workload": "hm_mount_global_matrices: HEX20 %dx%dx%d block, linear elastic skeleton, Biot 0.9, k 2.5e-3, "
                       "S 1e-4, gammaw 10, dt 0.05, base fixed, top drained; the whole call (device mount and CSC "
                       "export to host)" % n, "ndofs": nd, "nnz": int(G.nnz), "s": t, "value": nd / t,
           "unit": "DOF/s"}
    if with_cpu:
        import oracle as O
        from oracle import coupled as OC
        m2, e2, n2, p2 = _coupled_case(O, OC, (3, 2, 2))
        t0 = time.perf_counter()
        OC.mount_coupled(m2, OC.HYDRO, p2, e2, n2, 0.05, np.zeros(n2), gammaw=10.0)
        dt = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": n2 / dt, "unit": "DOF/s", "cores": 1, "kind": "port",
                               "sample": "oracle hm_mount_global_matrices (numpy) on HEX20 3x2x2, %d DOFs: %.2f s"
                                         % (n2, dt)}
    return out


def cpu_sample(nx, ny, nz, nthreads):
    """One linear increment of the same workload family on the CPU restatement: mount_K + direct solve
    (SuperLU) + update_state!.  Returns (ndofs, seconds)."""
    import oracle as O
    mesh = O.Mesh(O.Block([[0, 0, 0], [10.0, 4.0, 4.0]], nx=nx, ny=ny, nz=nz, cellshape=O.HEX20))
    ne = len(mesh.elems)
    E = np.exp(np.random.default_rng(SEED).normal(np.log(30e3), 0.3, ne))
    model = O.FEModel(mesh, [("all", O.LinearElastic(E=30e3, nu=0.2))], nips=27, elem_E=E)
    dofs, nu, setup = O.configure_dofs(model, [("z==0", O.SurfaceBC(ux=0, uy=0, uz=0)),
                                               ("z==4", O.SurfaceBC(tz=-1.0))])
    Uex, Fex = O.get_bc_vals(model, setup, len(dofs))
    t0 = time.perf_counter()
    K = O.mount_K(model, len(dofs), nthreads)
    U, F = Uex.copy(), Fex.copy()
    msg = O.solve_system(K, U, F, nu)
    assert msg is None, msg
    dF, msg = O.update_state(model, U, nthreads)
    assert msg is None, msg
    return len(dofs), time.perf_counter() - t0


CPU_TREND_MESH = (10, 4, 4)  # a second, smaller sample: the direct solve's DOF/s falls as the mesh grows


def cpu_baseline(a, steps, warmup):
    nx, ny, nz = dims(a.cpu_mesh)
    nth = os.cpu_count() or 1
    for _ in range(warmup):
        cpu_sample(nx, ny, nz, nth)
    ts = []
    for _ in range(max(steps, 1)):
        n, t = cpu_sample(nx, ny, nz, nth)
        ts.append(t)
    t = float(np.mean(ts))
    n2, t2 = cpu_sample(*CPU_TREND_MESH, nth)
    return {"value": n / t, "unit": "DOF/s", "cores": nth, "kind": "port",
            "sample": "HEX20 %dx%dx%d (%d DOFs) of the same block/load/E-field family, one linear increment: "
                      "mount_K (OpenMP, %d threads) + SuperLU direct solve (1 thread) + update_state!; %.2f s/step"
                      % (nx, ny, nz, n, nth, t),
            "note": "the reference (Julia) cannot run on this machine: this is the oracle's restatement of its CPU "
                    "path (C element kernels, scipy SuperLU in place of UMFPACK, one solver thread) on a mesh "
                    "with %dx fewer DOFs than the GPU workload's; a direct solve's DOF/s falls with size (trend)"
                    % max(1, round(2007483 / n)),
            "trend": [{"mesh": "%dx%dx%d" % CPU_TREND_MESH, "ndofs": n2, "dof_per_s": n2 / t2, "seconds": t2},
                      {"mesh": "%dx%dx%d" % (nx, ny, nz), "ndofs": n, "dof_per_s": n / t, "seconds": t}],
            "seconds_per_step": t}


def run_reference(a):
    rank, world = rank_info()
    if rank != 0:
        return None
    cb = cpu_baseline(a, a.steps, a.warmup)
    return {"metric": METRIC, "value": cb["value"], "unit": "DOF/s", "n_gpus": world, "steps": a.steps,
            "warmup": a.warmup, "ms_per_step": cb["seconds_per_step"] * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic", "impl": "reference",
            "config": {"workload": "HEX20 block 10x4x4 m, 27 IP, lognormal E (seed 0xA11A), nu=0.2, base fixed, top "
                                   "pressure 1.0; one linear increment (bounded CPU sample %s)" % a.cpu_mesh},
            "cpu_baseline": cb,
            "e2e": {"value": cb["value"], "unit": "DOF/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def amg_solve_only(a):
    """Profile driver: the bench workload at --mesh, assembled once, then --steps multigrid solves of it."""
    from amaru_gpu import _lib as L
    import torch
    model, Uex, Fex = workload_gpu(*dims(a.mesh))
    res = {"amg_solve_only": a.mesh}
    for smooth in (True, False):
        model.dev.set_amg_smoothing(smooth)
        out = []
        for rep in range(max(a.steps, 1) + 1):
            model.dev.assemble_K()  # a new K: the hierarchy's values are rebuilt by the solve
            torch.cuda.synchronize()
            t1 = time.perf_counter()
            _, _, st = model.dev.solve(Uex, Fex, L.default_solve_opts(method=L.SOLVER_AMG, rtol=1e-8))
            torch.cuda.synchronize()
            wall = time.perf_counter() - t1
            if rep > 0:  # the first solve also builds the hierarchy's structure on the host
                out.append({"s": st.seconds, "iterations": st.iterations, "rel_residual": st.rel_residual,
                            "wall_s": wall})
        res["smoothed" if smooth else "unsmoothed"] = out
    model.dev.set_amg_smoothing(True)
    return res


def main():
    a = parse()
    if a.amg_solve_only or a.batch_only:
        import torch
        torch.cuda.set_device(0)
        print(json.dumps(amg_solve_only(a) if a.amg_solve_only else batch_leg(a.batch_only)))
        return
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if world > 1:
        import torch.distributed as dist
        backend = "nccl" if a.impl == "ours" else "gloo"
        dist.init_process_group(backend)
    out = run_reference(a) if a.impl == "reference" else run_ours(a)
    rank, _ = rank_info()
    if rank == 0 and out is not None:
        print(json.dumps(out))
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
