#!/usr/bin/env python
"""Benchmark of the mechanical hot path on one GB300.

Workload: linear-elastic HEX20 block 10 x 4 x 4 m meshed 100 x 40 x 40
(669 161 nodes, 2 007 483 DOFs), 3x3x3 Gauss points, Young's modulus per
element lognormal(ln 30e3, 0.3) from a fixed seed, nu = 0.2, base z=0 fixed,
uniform pressure 1.0 on the top face.  A step is one linear load increment
of the staged Newton solver (mech_stage_solver!): device assembly of K (FP64
element integration + deterministic scatter), FP32 block-Jacobi PCG inside
FP64 iterative refinement to a relative residual of 1e-8, the internal-force
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
    return ap.parse_args()


def dims(s):
    return tuple(int(v) for v in s.lower().split("x"))


def rank_info():
    r = int(os.environ.get("RANK", "0"))
    w = int(os.environ.get("WORLD_SIZE", "1"))
    return r, w


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
    lin = L.default_solve_opts(method=L.SOLVER_MIXED, rtol=1e-8)
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
    t_step = max(times)
    if world > 1:
        import torch.distributed as dist
        tt = torch.tensor([t_step], device="cuda")
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        t_step = float(tt.item())
    mean_step = float(np.mean(times))
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
    achieved = spmv_b / spmv_t / 1e9
    traffic = None
    tp = os.path.join(ROOT, "profiles", "spmv32_traffic.json")
    if os.path.exists(tp):
        try:
            tj = json.load(open(tp))
            traffic = tj["bytes_per_block"] * sizes["nblocks"] + tj["bytes_per_node"] * sizes["nnodes"]
        except Exception:
            traffic = None

    # solve-only comparison: mixed-precision refined PCG vs the plain all-FP64 GPU path, same K and RHS
    solve_cmp = {}
    if not a.no_fp64:
        U0 = Uex.copy()
        F0 = Fex.copy()
        U1, F1, s_mixed = dev.solve(U0, F0, L.default_solve_opts(method=L.SOLVER_MIXED, rtol=1e-8))
        U2, F2, s_fp64 = dev.solve(U0, F0, L.default_solve_opts(method=L.SOLVER_FP64, rtol=1e-8, max_iters=200000))
        du = float(np.abs(U1[:model.nu] - U2[:model.nu]).max() / np.abs(U2[:model.nu]).max())
        solve_cmp = {"mixed_s": s_mixed.seconds, "mixed_iters": s_mixed.iterations,
                     "mixed_rel_residual": s_mixed.rel_residual, "fp64_s": s_fp64.seconds,
                     "fp64_iters": s_fp64.iterations, "fp64_rel_residual": s_fp64.rel_residual,
                     "speedup_vs_fp64": s_fp64.seconds / s_mixed.seconds, "max_rel_dU_mixed_vs_fp64": du}

    # e2e: the same step through the C ABI with host buffers (H2D inputs, D2H results inside)
    Uh = np.ascontiguousarray(Uex)
    Fh = np.ascontiguousarray(Fex)
    e2e_t = []
    for _ in range(a.steps):
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        rc, U, F, st = dev.stage_run(Uh, Fh, prm)
        torch.cuda.synchronize()
        e2e_t.append(time.perf_counter() - t1)
        if rc != 0:
            raise RuntimeError(dev.last_error())
    e2e_v = world * ndofs / float(np.mean(e2e_t))

    out = {
        "metric": METRIC, "value": value, "unit": "DOF/s", "n_gpus": world, "steps": a.steps, "warmup": a.warmup,
        "ms_per_step": mean_step * 1e3, "ms_per_step_max": t_step * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": "f64 assembly/residual/state, f32 Krylov", "data": "synthetic",
        "config": {"workload": "HEX20 %dx%dx%d block 10x4x4 m, 27 IP, lognormal E (seed 0xA11A), nu=0.2, base fixed, "
                               "top pressure 1.0; one linear increment: assemble K + PCG(f32)/IR(f64) to 1e-8 + "
                               "internal forces" % (nx, ny, nz),
                   "ndofs": ndofs, "nu": model.nu, "nnodes": sizes["nnodes"], "nelems": sizes["nelems"],
                   "nnz_blocks": sizes["nblocks"], "nnz": sizes["nblocks"] * 9,
                   "l2": "inputs larger than L2 (K32 %.2f GB, K64 %.2f GB)" % (sizes["nblocks"] * 36 / 1e9,
                                                                             sizes["nblocks"] * 72 / 1e9),
                   "parallelism": "replicas (one model per GPU)", "setup_s": setup_s},
        "solve": dict(solve_cmp, step_solve_s=float(np.mean(solve_s)), step_krylov_iters=int(np.mean(kry))),
        "roofline": {"bound": "hbm", "kernel": "k_spmv32 (FP32 BSR SpMV q = K p with fused p.q)",
                     "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                     "peak_source": peak_kind, "traffic": traffic, "bytes_per_launch": spmv_b,
                     "avg_launch_s": spmv_t,
                     "residual64": {"achieved": res_b / res_t / 1e9, "frac": res_b / res_t / 1e9 / hbm,
                                    "avg_launch_s": res_t}},
        "e2e": {"value": e2e_v, "unit": "DOF/s", "h2d_bytes_per_step": 2 * ndofs * 8, "d2h_bytes_per_step": 2 * ndofs * 8,
                "ms_per_step": float(np.mean(e2e_t)) * 1e3},
        "gpu_launches": launches,
        "clocks": clocks,
    }
    if rank == 0 and not a.no_cpu:
        out["cpu_baseline"] = cpu_baseline(a, steps=1, warmup=0)
    return out


# ---------------------------------------------------------------------------
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
    return {"value": n / t, "unit": "DOF/s", "cores": nth, "kind": "port",
            "sample": "HEX20 %dx%dx%d (%d DOFs) of the same block/load/E-field family, one linear increment: "
                      "mount_K (OpenMP, %d threads) + SuperLU direct solve (1 thread) + update_state!; %.2f s/step"
                      % (nx, ny, nz, n, nth, t),
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


def main():
    a = parse()
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
