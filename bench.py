"""Benchmark: element residual+Jacobian assembly throughput on GB300.

One step = one full residual + Jacobian assembly (Problem::get_jacobian) of
the workload: dof -> nodal-value scatter, the fused element kernel
(geometry + weak form + element matrices), and the deterministic scatter
into the CSR values and the residual.  Inputs are resident in HBM
(``value``); ``e2e`` repeats the step through the public API with the dof
vector copied in from pinned host memory and R + CSR values copied back.

Default workload: 2D steady incompressible Navier-Stokes, Taylor-Hood P2/P1
on a 256x256 split structured mesh (131,072 triangles), Re = 100, lid
u_x = 16x^2(1-x)^2, dofs perturbed by N(0, 1e-3); FP64 residual with FP64
Jacobian (headline) and FP32 Jacobian (variant).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                    [--workload ns|poisson|hex] [--size S]
"""
from __future__ import annotations

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

WORKLOADS = {
    # name: (description, default size)
    "ns": ("navier_stokes_th_p2p1_split_left_Re100", 256),
    "poisson": ("poisson_q2_quad_8gaussians", 64),
    "hex": ("nonlinear_diffusion_q2_hex_16gaussians", 48),
    "serving": ("serving_stream_poisson_ns_mixed", 64),
    "droplet": ("axisymmetric_droplet_ale_p2_stokes_free_surface_bdf2", 110),
}


def run_serving(args):
    """Serving stream: Poisson-process arrivals of Poisson / Navier-Stokes
    assemble+Newton requests, sides log-uniform in [16, --size], at each
    rate of --rates; the continuous-batching FP32-Jacobian server, and the
    plain FP64 one-request-at-a-time path on the first rate's stream."""
    import copy
    import torch
    from pyoomph_gb300 import serving as S
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    rates = [float(r) for r in args.rates.split(",")]
    workers = max(1, (os.cpu_count() or 2) - 2)
    # compile the four kernels (Poisson / NS x FP32 / FP64 Jacobian) before any clock starts
    for kind in ("poisson", "ns"):
        for prec in ("fp32", "fp64"):
            S._class_problem(kind, 8, prec, 1).initialise()
    per_rate = {}
    results = {}
    for rate in rates:
        reqs = S.make_stream(args.requests, rate=rate, seed=0, side_range=(16, args.size),
                             ns_side_max=args.ns_side_max)
        srv = S.Server(slots=4, jacobian_precision="fp32", workers=workers, device_solver=args.device_solver)
        if args.ns_device_min_side is not None:
            srv.device_saddle_min_side = args.ns_device_min_side
        t0 = time.perf_counter()
        done = srv.run(copy.deepcopy(reqs))
        wall = time.perf_counter() - t0
        sm = S.summary(done, wall)
        sm.update(wall_s=wall, assemblies=srv.assemblies, gpu_launches=srv.launches + srv.solver_launches,
                  mean_solve_s=srv.t_solve / max(1, sum(r.newton_iterations for r in done)),
                  device_solves=srv.device_solves)
        per_rate[str(rate)] = sm
        if rate == rates[0]:
            results["batched"] = {r.rid: r.dofs for r in done}
        srv.close()
    reqs = S.make_stream(args.requests, rate=rates[0], seed=0, side_range=(16, args.size),
                         ns_side_max=args.ns_side_max)
    t0 = time.perf_counter()
    seq = S.serve_sequential(copy.deepcopy(reqs), precision="fp64", device_solver=args.device_solver,
                             **({} if args.ns_device_min_side is None else
                                {"device_saddle_min_side": args.ns_device_min_side}))
    wall = time.perf_counter() - t0
    s_ = S.summary(seq, wall)
    s_["wall_s"] = wall
    err = max(float(np.max(np.abs(results["batched"][r.rid] - r.dofs)) / max(1.0, float(np.max(np.abs(r.dofs)))))
              for r in seq)
    head = per_rate[str(rates[min(1, len(rates) - 1)])]
    line = {"metric": "p50/p99 assemble+Newton request latency (serving stream)", "value": head["p50_s"],
            "unit": "s", "n_gpus": 1, "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64 residual, f32 Jacobian", "data": "synthetic",
            "config": {"workload": WORKLOADS["serving"][0], "requests": args.requests, "rates_per_s": rates,
                       "headline_rate_per_s": rates[min(1, len(rates) - 1)], "side_range": [16, args.size],
                       "ns_side_max": args.ns_side_max,
                       "slots_per_class": 4,
                       "linear_solver": (f"Poisson: native batched BiCGStab on the device; Navier-Stokes: SuperLU "
                                         f"(scipy) in {workers} worker processes below side "
                                         f"{args.ns_device_min_side or S.Server.default_saddle_min_side()}, "
                                         f"the device saddle-point GMRES (fieldsplit.py) from it")
                                        if args.device_solver else
                                        f"SuperLU (scipy), {workers} worker processes"},
            "batched_fp32_by_rate": per_rate, "sequential_fp64_at_first_rate": s_,
            "max_rel_solution_difference_batched_vs_sequential": err,
            "gpu_launches": sum(v["gpu_launches"] for v in per_rate.values())}
    print(json.dumps(line), flush=True)


def _peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d.get("hbm_gbs", 6800.0)), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc is not None:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() in ("active", "1"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def make_problem(workload: str, size: int, precision: str, epb=None, residual: str = "fp64"):
    from pyoomph_gb300 import workloads as W
    if workload == "ns":
        P = W.navier_stokes_problem(N=size, jacobian_precision=precision)
        P.elems_per_block = epb
        P.residual_precision = residual
        P.initialise()
        W.perturb_dofs(P, seed=0, sigma=1e-3)
    elif workload == "poisson":
        P = W.poisson_problem(N=size, seed=0, jacobian_precision=precision)
        P.elems_per_block = epb
        P.initialise()
    else:
        P = W.nonlinear_diffusion_problem(N=size, seed=0, jacobian_precision=precision)
        P.elems_per_block = epb
        P.initialise()
        x = np.random.default_rng(0).normal(0.0, 0.1, P.n_dof)
        P.set_dofs(x)
    return P


# elements per block measured fastest on GB300 where they differ from the
# generator's choice (threads follow: max(knots, ceil(rows / 2)) per element)
TUNED_EPB = {("ns", 256, "df64"): 32, ("ns", 256, "df64:df64"): 32, ("ns", 256, "fp32:df64"): 24}

# DRAM bytes (read + write) per launch of an element kernel, keyed by the
# generated kernel's name (its source hash): dram__bytes_read.sum +
# dram__bytes_write.sum from one ncu capture of that exact kernel, scaled
# from the captured mesh to the bench's by element count
# (profiles/dram_traffic_element_kernels.md gives the commands).  A kernel
# with no capture reports null.  Value: (bytes per element, elements of the
# captured launch).
MEASURED_TRAFFIC = {
    # NS Taylor-Hood 256^2, FP64 (32 elements and 256 threads per block):
    # 16,544,512 read + 196,024,832 written
    "fe_elem_p2_tri_f64_aff_7785240288": ((16544512 + 196024832) / 131072, 131072),
}


def measured_traffic(kernel_name: str, n_elem: int):
    t = MEASURED_TRAFFIC.get(kernel_name)
    if t is None:
        return None
    bytes_per_elem, captured_elems = t
    return {"bytes": bytes_per_elem * n_elem, "kernel": kernel_name, "captured_n_elem": captured_elems,
            "scaled_to_n_elem": n_elem}


def element_algorithmic_bytes(P) -> int:
    """Compulsory HBM bytes of one element-kernel launch: connectivity,
    nodal positions and values read once, element residuals and matrices
    written once (tables are negligible)."""
    m = P.mesh
    nl = P.kernel.layout.n
    jb = 8 if P._prec == "f64" else 4
    return int(m.n_elem * m.etype.nnode * 4 + m.n_nodes * m.dim * 8 + m.n_nodes * len(P.fields) * 8
               + m.n_elem * nl * 8 + m.n_elem * nl * nl * jb)


def fp64_peak_tflops(torch) -> float:
    """FP64 denominator measured in this run: cuBLAS DGEMM 4096^3, best of 5."""
    n = 4096
    a = torch.randn(n, n, dtype=torch.float64, device="cuda")
    b = torch.randn(n, n, dtype=torch.float64, device="cuda")
    for _ in range(2):
        a @ b
    torch.cuda.synchronize()
    best = float("inf")
    for _ in range(5):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        a @ b
        e1.record()
        torch.cuda.synchronize()
        best = min(best, e0.elapsed_time(e1) / 1e3)
    del a, b
    return 2.0 * n ** 3 / best / 1e12


def time_steps(torch, fn, steps: int, warmup: int):
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    st = torch.cuda.current_stream()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(st)
    for _ in range(steps):
        fn()
    e1.record(st)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / steps


def run_gb300(args):
    import torch
    from pyoomph_gb300 import problem as _p  # noqa: F401
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    hbm_peak, peak_kind = _peaks()
    results = {}
    tuned = {}
    for prec in ("fp64", "fp32", "df64"):
        # launch shapes --autotune measured fastest on GB300 where they differ
        # from the generator's default (NS 256^2 df64: 48 elements/block
        # 1.04 ms, default 46: 1.10 ms -- whole waves of 152 blocks)
        epb = TUNED_EPB.get((args.workload, args.size, prec))
        if args.autotune:
            from pyoomph_gb300 import autotune as AT
            P0 = make_problem(args.workload, args.size, prec)
            cands = AT.epb_candidates(P0.mesh.etype.nq, P0.kernel.layout.n)
            key = f"{args.workload}-{args.size}-{prec}-{P0.kernel.name}"
            del P0
            epb, table = AT.tune(key, lambda e: make_problem(args.workload, args.size, prec, e), cands,
                                 use_cache=False)
            tuned[prec] = {"elems_per_block": epb, "ms_per_assembly": table}
        P = make_problem(args.workload, args.size, prec, epb)
        P.check()
        asm = lambda: P.assemble_device(with_jacobian=True)
        # device-resident throughput
        for _ in range(args.warmup):
            asm()
        torch.cuda.synchronize()
        if dist is not None:
            dist.barrier()
        with ClockSampler(local) as cs:
            ms = time_steps(torch, asm, args.steps, 0)
        if dist is not None:
            t = torch.tensor([ms], device="cuda")
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            ms = float(t.item())
        P.check()
        # stage breakdown (element kernel = dominant kernel)
        P.set_stage_timing(True)
        for _ in range(max(3, min(args.steps, 10))):
            asm()
        stage_ms, calls = P.stage_times()
        P.set_stage_timing(False)
        stage_ms = stage_ms / max(calls, 1)
        # end to end through the public API with host buffers
        xh = torch.from_numpy(P.get_dofs()).pin_memory()
        Rh = torch.empty(P.n_dof, dtype=torch.float64).pin_memory()
        Jh = torch.empty(P.nnz, dtype=P.J_dev.dtype).pin_memory()

        def e2e_plain():
            P.x_dev.copy_(xh, non_blocking=True)
            P.assemble_device(with_jacobian=True)
            Rh.copy_(P.R_dev[:P.n_dof], non_blocking=True)
            Jh.copy_(P.J_dev[:P.nnz], non_blocking=True)

        ms_e2e_plain = time_steps(torch, e2e_plain, max(3, args.steps), args.warmup)
        # public host-buffer API: dofs in, R and CSR values out, with the copies
        # of finished rows overlapping the element chunks still running; the
        # chunk count (rounded to whole waves by the library) is chosen by timing
        e2e_by_chunks = {}
        for nc in (2, 4, 8, 16):
            e2e_by_chunks[nc] = time_steps(torch, lambda: P.assemble_host(xh, Rh, Jh, True, chunks=nc),
                                           max(3, args.steps), args.warmup)
        chunks = min(e2e_by_chunks, key=e2e_by_chunks.get)
        ms_e2e = e2e_by_chunks[chunks]
        torch.cuda.synchronize()
        P.check()
        # the reference's default value-dependent pattern (zero filter at 0.0)
        # on the same state: the filtered gather and compaction replace the
        # structural gather
        zf = None
        if prec == "fp64":
            ms_zf = time_steps(torch, lambda: P.assemble_device(with_jacobian=True, zero_threshold=0.0),
                               args.steps, args.warmup)
            P.check()
            nnz_zf = P.assemble_filtered(0.0)[2].size
            zf = {"ms_per_step": ms_zf, "nnz": int(nnz_zf), "structural_nnz": int(P.nnz),
                  "launches_per_step": P.launch_count(True, zero_filter=True)}
        # the same assembly replayed as one CUDA graph
        P.capture_assembly(with_jacobian=True)
        ms_graph = time_steps(torch, P.assemble_graph, args.steps, args.warmup)
        P.check()
        results[prec] = dict(P=P, ms=ms, stage_ms=stage_ms, ms_e2e=ms_e2e, clocks=cs.summary(), ms_graph=ms_graph, zf=zf,
                             ms_e2e_plain=ms_e2e_plain, e2e_chunks=chunks, e2e_by_chunks=e2e_by_chunks,
                             h2d=int(P.n_dof * 8), d2h=int(P.n_dof * 8 + P.nnz * P.J_dev.element_size()))
    if args.workload == "ns":
        # the FP32 and df64 Jacobians with the residual path in double-float
        # (residual_precision="df64"): device steps, stages, graph replay and
        # the host-buffer API at the chunk count chosen above for the same
        # Jacobian precision
        for prec in ("fp32:df64", "df64:df64"):
            jp, _, rp = prec.partition(":")
            P = make_problem(args.workload, args.size, jp, TUNED_EPB.get((args.workload, args.size, prec)), rp)
            asm = lambda: P.assemble_device(with_jacobian=True)
            ms = time_steps(torch, asm, args.steps, args.warmup)
            if dist is not None:
                t = torch.tensor([ms], device="cuda")
                dist.all_reduce(t, op=dist.ReduceOp.MAX)
                ms = float(t.item())
            P.set_stage_timing(True)
            for _ in range(max(3, min(args.steps, 10))):
                asm()
            stage_ms, calls = P.stage_times()
            P.set_stage_timing(False)
            xh = torch.from_numpy(P.get_dofs()).pin_memory()
            Rh = torch.empty(P.n_dof, dtype=torch.float64).pin_memory()
            Jh = torch.empty(P.nnz, dtype=P.J_dev.dtype).pin_memory()
            chunks = results[jp]["e2e_chunks"]
            ms_e2e = time_steps(torch, lambda: P.assemble_host(xh, Rh, Jh, True, chunks=chunks),
                                max(3, args.steps), args.warmup)
            P.capture_assembly(with_jacobian=True)
            ms_graph = time_steps(torch, P.assemble_graph, args.steps, args.warmup)
            P.check()
            results[prec] = dict(P=P, ms=ms, stage_ms=stage_ms / max(calls, 1), ms_e2e=ms_e2e, ms_graph=ms_graph,
                                 e2e_chunks=chunks, h2d=int(P.n_dof * 8),
                                 d2h=int(P.n_dof * 8 + P.nnz * P.J_dev.element_size()))
    from pyoomph_gb300.codegen import estimate_flops
    peak64 = fp64_peak_tflops(torch)
    main = results["fp64"]
    P = main["P"]
    n_elem = P.mesh.n_elem
    value = n_elem * world / (main["ms"] / 1e3)
    elem_ms = float(main["stage_ms"][1])
    abytes = element_algorithmic_bytes(P)
    achieved = abytes / (elem_ms / 1e3) / 1e9
    launches = P.launch_count(True)
    line = {
        "metric": "element residual+Jacobian assemblies/s (full CSR assembly)",
        "value": value,
        "unit": "elements/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": main["ms"],
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic",
        "config": {"workload": WORKLOADS[args.workload][0], "mesh_side": args.size, "n_elem": n_elem,
                   "n_dof": P.n_dof, "nnz": P.nnz, "jacobian": "fp64", "residual": "fp64",
                   "l2": "working set per step > L2 (element matrices + CSR + contribution lists)",
                   "parallelism": "replicas" if world > 1 else "single-gpu"},
        "assemblies_per_s": 1e3 / main["ms"],
        "stage_ms": {"dof_scatter": float(main["stage_ms"][0]), "element_kernel": elem_ms,
                     "residual_gather": float(main["stage_ms"][2]), "jacobian_gather": float(main["stage_ms"][3])},
        "roofline": {"bound": "hbm", "kernel": P.kernel.name, "achieved": achieved, "peak": hbm_peak,
                     "unit": "GB/s", "frac": achieved / hbm_peak, "peak_kind": peak_kind,
                     "algorithmic_bytes_per_launch": abytes,
                     "traffic": (measured_traffic(P.kernel.name, n_elem) or {}).get("bytes"),
                     "traffic_capture": measured_traffic(P.kernel.name, n_elem)},
        "compute_roofline": {"pipe": "fp64", "kernel": P.kernel.name,
                             "flops_per_element": estimate_flops(P.kernel, P.affine)["fp64"],
                             "achieved": estimate_flops(P.kernel, P.affine)["fp64"] * n_elem / (elem_ms / 1e3) / 1e12,
                             "peak": peak64, "unit": "TFLOP/s",
                             "frac": estimate_flops(P.kernel, P.affine)["fp64"] * n_elem / (elem_ms / 1e3) / 1e12 / peak64,
                             "peak_kind": "measured in this run: cuBLAS DGEMM 4096^3 (torch.matmul float64)",
                             "flops": "counted from the generated kernel's operation structure, FMA = 2"},
        "e2e": {"value": n_elem * world / (main["ms_e2e"] / 1e3), "unit": "elements/s",
                "h2d_bytes_per_step": main["h2d"], "d2h_bytes_per_step": main["d2h"],
                "ms_per_step": main["ms_e2e"], "api": "Problem.assemble_host (fe_assemble_pipelined)",
                "chunks_requested": main["e2e_chunks"],
                "ms_by_chunks": {str(k): v for k, v in main["e2e_by_chunks"].items()},
                "unpipelined_ms_per_step": main["ms_e2e_plain"]},
        "gpu_launches": launches * args.steps,
        "clocks": main["clocks"],
        "cuda_graph": {"ms_per_step": main["ms_graph"], "value": n_elem * world / (main["ms_graph"] / 1e3),
                       "launches_per_step": 1},
        "zero_filter": dict(main["zf"], what="the reference's default sparse assembly: oomph's zero filter at "
                            "0.0, value-dependent CSR pattern compacted on the device (FE_ASSEMBLE_ZERO_FILTER)"),
        "launch_shape": {"elems_per_block": P.kernel.epb, "threads": P.kernel.threads,
                         "smem_bytes": P.kernel.smem_bytes, "min_blocks_per_sm": P.kernel.min_blocks or None,
                         "autotuned": tuned or None},
    }
    r32 = results["fp32"]
    f32 = estimate_flops(r32["P"].kernel, r32["P"].affine)
    line["fp32_jacobian"] = {"value": n_elem * world / (r32["ms"] / 1e3), "unit": "elements/s",
                             "ms_per_step": r32["ms"], "element_kernel_ms": float(r32["stage_ms"][1]),
                             "fp64_tflops": f32["fp64"] * n_elem / (float(r32["stage_ms"][1]) / 1e3) / 1e12,
                             "fp32_tflops": f32["jac"] * n_elem / (float(r32["stage_ms"][1]) / 1e3) / 1e12,
                             "e2e": {"value": n_elem * world / (r32["ms_e2e"] / 1e3),
                                     "h2d_bytes_per_step": r32["h2d"], "d2h_bytes_per_step": r32["d2h"]},
                             "cuda_graph_ms_per_step": r32["ms_graph"],
                             "elems_per_block": r32["P"].kernel.epb}
    rdf = results["df64"]
    fdf = estimate_flops(rdf["P"].kernel, rdf["P"].affine)
    kdf = float(rdf["stage_ms"][1]) / 1e3
    # full-size parity of the double-float Jacobian against the FP64 one (same
    # state, same pattern): max |J_df64 - J_fp64| / max |J_fp64|
    Pdf = rdf["P"]
    Pdf.assemble_device(with_jacobian=True)
    P.assemble_device(with_jacobian=True)
    jdiff = float((Pdf.J_dev[:P.nnz] - P.J_dev[:P.nnz]).abs().max() / P.J_dev[:P.nnz].abs().max())
    rdiff = float((Pdf.R_dev[:P.n_dof] - P.R_dev[:P.n_dof]).abs().max() / P.R_dev[:P.n_dof].abs().max())
    line["df64_jacobian"] = {
        "what": "FP64 residual and FP64 Jacobian values; the Jacobian's contraction (phase B) in double-float "
                "(hi + lo pairs of FP32, ~2^-48 relative per operation) on the FP32 pipes",
        "value": n_elem * world / (rdf["ms"] / 1e3), "unit": "elements/s", "ms_per_step": rdf["ms"],
        "element_kernel_ms": kdf * 1e3, "kernel": Pdf.kernel.name,
        "fp64_tflops": fdf["fp64"] * n_elem / kdf / 1e12,
        "df64_contraction_tflops_fp64_equivalent": fdf.get("df64", 0.0) * n_elem / kdf / 1e12,
        "max_rel_jacobian_difference_vs_fp64": jdiff, "max_rel_residual_difference_vs_fp64": rdiff,
        "e2e": {"value": n_elem * world / (rdf["ms_e2e"] / 1e3), "unit": "elements/s",
                "h2d_bytes_per_step": rdf["h2d"], "d2h_bytes_per_step": rdf["d2h"], "ms_per_step": rdf["ms_e2e"]},
        "cuda_graph_ms_per_step": rdf["ms_graph"], "elems_per_block": Pdf.kernel.epb,
        "threads": Pdf.kernel.threads, "smem_bytes": Pdf.kernel.smem_bytes}
    for jp, key in (("fp32", "fp32_jacobian"), ("df64", "df64_jacobian")):
        r = results.get(f"{jp}:df64")
        if r is None:
            continue
        kms = float(r["stage_ms"][1])
        fr = estimate_flops(r["P"].kernel, r["P"].affine)
        line[key]["df64_residual"] = {
            "what": "the same Jacobian with the residual path (interpolation from FP64 differences to node 0, "
                    "pointwise residual, pull-back, test-function contraction) in double-float on the FP32 "
                    "pipes: Problem.residual_precision = 'df64'",
            "value": n_elem * world / (r["ms"] / 1e3), "unit": "elements/s", "ms_per_step": r["ms"],
            "element_kernel_ms": kms, "kernel": r["P"].kernel.name,
            "stage_ms": {"dof_scatter": float(r["stage_ms"][0]), "element_kernel": kms,
                         "residual_gather": float(r["stage_ms"][2]), "jacobian_gather": float(r["stage_ms"][3])},
            "fp64_flops_per_element": fr["fp64"], "df64_residual_flops_per_element": fr["df64_residual"],
            "e2e": {"value": n_elem * world / (r["ms_e2e"] / 1e3), "unit": "elements/s",
                    "ms_per_step": r["ms_e2e"], "chunks_requested": r["e2e_chunks"],
                    "h2d_bytes_per_step": r["h2d"], "d2h_bytes_per_step": r["d2h"]},
            "cuda_graph_ms_per_step": r["ms_graph"], "elems_per_block": r["P"].kernel.epb,
            "threads": r["P"].kernel.threads, "smem_bytes": r["P"].kernel.smem_bytes}
    if args.workload in ("hex", "poisson") and world == 1:
        # a whole Newton solve on the device (assembly + BiCGStab on the resident
        # Jacobian), from the zero initial guess to max |R| < 1e-10; a small
        # solve first loads the vector kernels the solver uses
        for prec in ("fp64", "fp32"):
            PW = make_problem(args.workload, 4, prec)
            PW.linear_solver = "bicgstab"
            PW.solve()
            del PW
        for prec in ("fp64", "fp32"):
            PN = make_problem(args.workload, args.size, prec)
            PN.set_dofs(np.zeros(PN.n_dof))
            PN.linear_solver = "bicgstab"
            PN.newton_solver_tolerance = 1e-10
            PN.max_newton_iterations = 20
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            hist = PN.solve()
            torch.cuda.synchronize()
            t_solve = time.perf_counter() - t0
            kinfo = PN._krylov.info()
            # the CSR SpMV alone on the converged Jacobian: algorithmic bytes =
            # values + column indices + row pointers + x + y, once
            from pyoomph_gb300.linsolve import DeviceCSR
            A = DeviceCSR.of_problem(PN)
            xs = torch.ones(PN.n_dof, dtype=torch.float64, device="cuda")
            ys = torch.empty_like(xs)
            st = torch.cuda.current_stream().cuda_stream

            def time_spmv(fn, reps=20):
                for _ in range(3):
                    fn()
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record()
                for _ in range(reps):
                    fn()
                e1.record()
                torch.cuda.synchronize()
                return e0.elapsed_time(e1) / reps
            spmv_ms = time_spmv(lambda: PN._krylov.matvec(xs, ys))          # through the solver (fe_krylov_matvec)
            spmv_rows_ms = time_spmv(lambda: A.matvec(xs, ys, st))           # fe_csr_spmv directly
            jb = 8 if prec == "fp64" else 4
            spmv_bytes = PN.nnz * (jb + 4) + (PN.n_dof + 1) * 4 + 2 * PN.n_dof * 8
            kits = PN.timings.get("krylov_iterations") or 0
            line.setdefault("newton_device_solve", {})[prec] = {
                "s": t_solve, "n_dof": PN.n_dof, "newton_iterations": len(hist) - 1,
                "krylov_iterations": kits, "residuals": hist,
                "linear_solve_s": PN.timings.get("newton_linear_solve_s"),
                "ms_per_krylov_iteration": (1e3 * PN.timings["newton_linear_solve_s"] / kits) if kits else None,
                "solver_launches": kinfo["launches"], "solver_graph_replays": kinfo["graph_replays"],
                "spmv": {"kernel": "k_csr_spmv (fe_krylov_matvec)", "ms": spmv_ms,
                         "algorithmic_bytes": spmv_bytes, "gbs": spmv_bytes / spmv_ms / 1e6,
                         "fe_csr_spmv_ms": spmv_rows_ms,
                         "frac_of_hbm": spmv_bytes / spmv_ms / 1e6 / hbm_peak if hbm_peak else None,
                         "l2": "matrix > L2 (streamed once per product)" if spmv_bytes > 129e6 else
                               "matrix fits in L2 (warm repeats)"},
                "linear_solver": "native batched Jacobi-BiCGStab (fe_krylov_solve: fe_csr_spmv + fused "
                                 "vector kernels, CUDA-graph blocks of 8 iterations)"}
            del PN, A
    if args.workload == "ns" and world == 1:
        # the whole Newton solve of the Navier-Stokes problem on the device
        # (fieldsplit.py: GMRES with the block-triangular multigrid
        # preconditioner) from the perturbed state to max |R| < 1e-10, with
        # the FP64 and the FP32 Jacobian; a small solve first loads the kernels
        PW = make_problem("ns", 8, "fp64")
        PW.linear_solver = "fieldsplit"
        PW.solve()
        del PW
        sols = {}
        for prec in ("fp64", "fp32"):
            PN = make_problem("ns", args.size, prec)
            PN.linear_solver = "fieldsplit"
            PN.newton_solver_tolerance = 1e-10
            PN.max_newton_iterations = 30
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            PN.assemble_device(with_jacobian=True)
            PN._fieldsplit_solver().setup()          # the multigrid hierarchy (host, once per mesh)
            t_setup = time.perf_counter() - t0
            t0 = time.perf_counter()
            hist = PN.solve()
            torch.cuda.synchronize()
            t_solve = time.perf_counter() - t0
            sols[prec] = PN.get_dofs()
            line.setdefault("newton_device_solve", {})[prec] = {
                "s": t_solve, "preconditioner_setup_s": t_setup, "n_dof": PN.n_dof,
                "newton_iterations": len(hist) - 1, "residuals": hist,
                "krylov_iterations": PN.timings.get("krylov_iterations"),
                "linear_solve_s": PN.timings.get("newton_linear_solve_s"),
                "multigrid_levels": PN._fieldsplit.sizes,
                "linear_solver": "GMRES(60), block upper-triangular preconditioner: smoothed-aggregation V-cycle "
                                 "on the velocity block, lumped pressure mass / viscosity for the Schur complement "
                                 "(fieldsplit.py)"}
            del PN
        line["newton_device_solve"]["max_rel_solution_difference_fp32_vs_fp64_jacobian"] = float(
            np.max(np.abs(sols["fp32"] - sols["fp64"])) / np.max(np.abs(sols["fp64"])))
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        # the checker, after every timed region
        line["parity"] = parity_vs_oracle(args, results)
        if "fp32" in line["parity"]:
            line["fp32_jacobian"]["max_rel_jacobian_error_vs_fp64_oracle"] = line["parity"]["fp32"].get("max_rel_J")
        for jp, key in (("fp32", "fp32_jacobian"), ("df64", "df64_jacobian")):
            par = line["parity"].get(f"{jp}:df64")
            if par and "df64_residual" in line[key]:
                line[key]["df64_residual"]["max_rel_residual_error_vs_oracle"] = par.get("max_rel_R")
                line[key]["df64_residual"]["max_rel_jacobian_error_vs_oracle"] = par.get("max_rel_J")
    if rank == 0 and world == 1 and args.workload == "ns" and not args.no_extras:
        # the other benchmark workloads, measured in this same run (after
        # the headline's timed regions): Poisson Q2 64^2, the Q2 hex 48^3
        # (FP32 Jacobian on the tensor cores), the moving-mesh droplet and a
        # bounded serving stream
        extras = {}
        for wl in ("poisson", "hex"):
            extras[wl] = measure_extra(wl, WORKLOADS[wl][1], args.steps, args.warmup, hbm_peak, peak64)
        extras["droplet"] = measure_droplet_compact(WORKLOADS["droplet"][1], args.steps, args.warmup, hbm_peak,
                                                    peak64)
        extras["serving"] = measure_serving_bounded()
        line["other_workloads"] = extras
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(args, threads=1)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


def measure_extra(workload: str, size: int, steps: int, warmup: int, hbm_peak: float, peak64: float,
                  with_parity: bool = True):
    """A compact record of another workload in the same run: per Jacobian
    precision the device-resident step, the element kernel (and, for the
    tensor-core contraction, its own kernel), the end-to-end step through
    the host-buffer API, flop rates; full-size parity against the oracle;
    for Poisson and the hex the whole Newton solve on the device."""
    import torch
    from types import SimpleNamespace
    from pyoomph_gb300.codegen import estimate_flops
    out = {"workload": WORKLOADS[workload][0], "mesh_side": size}
    results = {}
    for prec in ("fp64", "fp32", "df64"):
        P = make_problem(workload, size, prec)
        E = P.mesh.n_elem
        asm = lambda: P.assemble_device(with_jacobian=True)
        ms = time_steps(torch, asm, steps, warmup)
        P.check()
        P.set_stage_timing(True)
        for _ in range(5):
            asm()
        st, calls = P.stage_times()
        P.set_stage_timing(False)
        st = st / max(calls, 1)
        xh = torch.from_numpy(P.get_dofs()).pin_memory()
        Rh = torch.empty(P.n_dof, dtype=torch.float64).pin_memory()
        Jh = torch.empty(P.nnz, dtype=P.J_dev.dtype).pin_memory()
        ms_e2e = time_steps(torch, lambda: P.assemble_host(xh, Rh, Jh, True, chunks=4), steps, warmup)
        P.check()
        fl = estimate_flops(P.kernel, P.affine)
        d = {"ms_per_step": ms, "value": E / (ms / 1e3), "unit": "elements/s", "kernel": P.kernel.name,
             "element_kernel_ms": float(st[1]), "jacobian_gather_ms": float(st[3]),
             "e2e": {"value": E / (ms_e2e / 1e3), "ms_per_step": ms_e2e, "h2d_bytes_per_step": int(P.n_dof * 8),
                     "d2h_bytes_per_step": int(P.n_dof * 8 + P.nnz * P.J_dev.element_size()),
                     "api": "Problem.assemble_host (fe_assemble_pipelined)"},
             "fp64_tflops": fl["fp64"] * E / (float(st[1]) / 1e3) / 1e12,
             "fp64_frac_of_dgemm": fl["fp64"] * E / (float(st[1]) / 1e3) / 1e12 / peak64,
             "roofline_hbm_frac": element_algorithmic_bytes(P) / (float(st[1]) / 1e3) / 1e9 / hbm_peak}
        if P.kernel.tc_pairs:
            d["tensor_cores"] = {
                "kernel": "k_tc_contract (tcgen05.mma kind::tf32, 3xTF32 split)",
                "ms": float(st[4]), "useful_tflops": fl["tensor"] * E / (float(st[4]) / 1e3) / 1e12,
                "issued_tflops": fl["tensor_issued"] * E / 4 / (float(st[4]) / 1e3) / 1e12,
                "useful_flops_per_element": fl["tensor"]}
        results[prec] = {"P": P}
        out[prec] = d
    n_elem = results["fp64"]["P"].mesh.n_elem
    out.update(n_elem=n_elem, n_dof=results["fp64"]["P"].n_dof, nnz=results["fp64"]["P"].nnz)
    if with_parity:
        out["parity"] = parity_vs_oracle(SimpleNamespace(workload=workload, size=size), results)
    for r in results.values():
        del r["P"]
    if workload in ("hex", "poisson"):
        out["newton_device_solve"] = {}
        for prec in ("fp64", "fp32"):
            PN = make_problem(workload, size, prec)
            PN.set_dofs(np.zeros(PN.n_dof))
            PN.linear_solver = "bicgstab"
            PN.newton_solver_tolerance = 1e-10
            PN.max_newton_iterations = 20
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            hist = PN.solve()
            torch.cuda.synchronize()
            out["newton_device_solve"][prec] = {
                "s": time.perf_counter() - t0, "newton_iterations": len(hist) - 1, "residuals": hist,
                "krylov_iterations": PN.timings.get("krylov_iterations")}
            del PN
    return out


def measure_serving_bounded(requests: int = 200, rate: float = 50.0, side_max: int = 64, seq_requests: int = 40):
    """A bounded serving stream: Poisson-process arrivals of Poisson and
    Navier-Stokes assemble+Newton requests (sides log-uniform in
    [16, side_max]) through the continuous-batching FP32-Jacobian server
    (Poisson Newton systems solved on the device by the batched BiCGStab;
    Navier-Stokes ones by SuperLU in worker processes below the server's
    device_saddle_min_side, by the device saddle-point GMRES from it), and
    the plain FP64 one-request-at-a-time path on
    the first seq_requests of the same stream."""
    import copy
    from pyoomph_gb300 import serving as S
    workers = max(1, (os.cpu_count() or 2) - 2)
    for kind in ("poisson", "ns"):
        for prec in ("fp32", "fp64"):
            S._class_problem(kind, 8, prec, 1).initialise()
    reqs = S.make_stream(requests, rate=rate, seed=0, side_range=(16, side_max), ns_side_max=side_max)
    srv = S.Server(slots=4, jacobian_precision="fp32", workers=workers, device_solver=True)
    t0 = time.perf_counter()
    done = srv.run(copy.deepcopy(reqs))
    wall = time.perf_counter() - t0
    out = {"requests": requests, "rate_per_s": rate, "side_range": [16, side_max], "wall_s": wall,
           "batched_fp32": S.summary(done, wall), "assemblies": srv.assemblies,
           "gpu_launches": srv.launches + srv.solver_launches, "device_solves": srv.device_solves,
           "linear_solver": f"Poisson: native batched BiCGStab on the device; Navier-Stokes: SuperLU in "
                            f"{workers} worker processes below side {srv.device_saddle_min_side}, the device "
                            f"saddle-point GMRES (fieldsplit.py) from it"}
    srv.close()
    sub = copy.deepcopy(reqs[:seq_requests])
    t0 = time.perf_counter()
    seq = S.serve_sequential(sub, precision="fp64", device_solver=True)
    wall2 = time.perf_counter() - t0
    out["sequential_fp64_first_requests"] = dict(S.summary(seq, wall2), requests=seq_requests)
    by = {r.rid: r for r in done}
    ok = [r for r in seq if r.error is None and by[r.rid].error is None]
    out["max_rel_solution_difference_batched_vs_sequential"] = max(
        [float(np.max(np.abs(by[r.rid].dofs - r.dofs)) / max(1.0, float(np.max(np.abs(r.dofs))))) for r in ok],
        default=None)
    out["requests_compared"] = len(ok)
    return out


def _oracle_problem(workload: str, side: int):
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    from pyoomph_gb300.workloads import draw_gaussians
    if workload == "ns":
        m = O.mesh(O.P2_TRI, side, side)
        OP = O.navier_stokes_problem(m, rho=1.0, mu=0.01)
        OP.set_dofs(OP.dofs() + np.random.default_rng(0).normal(0.0, 1e-3, OP.n_dof))
    elif workload == "poisson":
        OP = O.poisson_problem(O.mesh(O.Q2_QUAD, side, side), draw_gaussians(0, 8, 2))
    else:
        OP = O.poisson_problem(O.mesh(O.Q2_HEX, side, side, side), draw_gaussians(0, 16, 3),
                               eq=O.EQ_NONLINEAR_DIFFUSION)
    return OP


def _sample_side(workload: str, size: int) -> int:
    """The side the CPU baseline times: the bench's own side where one
    assembly takes a few seconds on a host core (NS 256^2: ~2.5 s), a
    smaller cube for the hex (48^3: ~15 s per assembly)."""
    return {"ns": size, "poisson": size, "hex": min(size, 24)}[workload]


_CPU = None


def _cpu_init(workload: str, side: int):
    """Pool initialiser: the oracle built with pyoomph's JIT flags, the
    problem, one warm-up assembly."""
    global _CPU
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    flags = O.use_jit_flags_build()
    OP = _oracle_problem(workload, side)
    O.assemble(OP, True, 0.0)
    _CPU = (O, OP, flags)


def _cpu_time(seconds: float):
    """Whole assemblies (the reference's default zero filter, threshold 0)
    until `seconds` have passed; at least one."""
    O, OP, flags = _CPU
    n_elem = OP.mesh.conn.shape[0]
    t0 = time.perf_counter()
    done = 0
    while True:
        O.assemble(OP, True, 0.0)
        done += 1
        if time.perf_counter() - t0 >= seconds:
            break
    return n_elem * done, time.perf_counter() - t0, done, flags


class CpuPool:
    """`threads` spawned processes, each holding the oracle problem."""

    def __init__(self, workload: str, side: int, threads: int):
        import multiprocessing as mp
        self.threads = threads
        self.pool = mp.get_context("spawn").Pool(threads, initializer=_cpu_init, initargs=(workload, side))

    def measure(self, seconds: float):
        res = self.pool.map(_cpu_time, [seconds] * self.threads)
        return sum(r[0] / r[1] for r in res), sum(r[2] for r in res), res[0][3]

    def close(self):
        self.pool.close()
        self.pool.join()


def _cpu_sample_text(workload, side, n, seconds, flags, threads):
    return (f"{WORKLOADS[workload][0]} side {side}, {n} full assemblies in ~{seconds:.0f} s on {threads} "
            f"core(s) (oracle/fe_oracle.c: restated element code and vectors-of-pairs assembly with the "
            f"default zero filter, compiled {flags})")


def cpu_baseline(args, threads: int = 1, seconds: float = 10.0):
    """The oracle's restated reference assembly (vectors-of-pairs, restated
    element code, pyoomph's JIT flags) timed on the host cores on a bounded
    sample: whole assemblies of the bench's mesh (hex: a 24^3 cube)."""
    side = _sample_side(args.workload, args.size)
    pool = CpuPool(args.workload, side, threads)
    try:
        value, n, flags = pool.measure(seconds)
    finally:
        pool.close()
    return {"value": value, "unit": "elements/s", "cores": threads, "kind": "port", "mesh_side": side,
            "sample": _cpu_sample_text(args.workload, side, n, seconds, flags, threads)}


def parity_vs_oracle(args, results):
    """Full-size parity of this run's assemblies: the oracle assembles the
    bench's mesh on the same dof vector once (structural pattern, oomph's
    threshold -1); every precision's R and CSR J are compared with it."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    P = results["fp64"]["P"]
    OP = _oracle_problem(args.workload, args.size)
    if not np.array_equal(P.eqn, OP.eqn):
        return {"vs": "oracle", "size": args.size, "error": "equation numbering differs"}
    OP.set_dofs(P.get_dofs())
    t0 = time.perf_counter()
    R0, rp, ci, v = O.assemble(OP, True, -1.0)
    out = {"vs": "oracle (oracle/fe_oracle.c, vectors-of-pairs, structural pattern)", "size": args.size,
           "oracle_assembly_s": time.perf_counter() - t0}
    nR = max(float(np.max(np.abs(R0))), 1e-300)
    nJ = max(float(np.max(np.abs(v))), 1e-300)
    for prec, r in results.items():
        Q = r["P"]
        if not np.array_equal(Q.get_dofs(), OP.dofs()):
            out[prec] = {"error": "dof vector differs from the oracle's"}
            continue
        R, J = Q.get_jacobian()
        out[prec] = {"pattern_bit_exact": bool(np.array_equal(J.indptr, rp) and np.array_equal(J.indices, ci)),
                     "max_rel_R": float(np.max(np.abs(R - R0)) / nR),
                     "max_rel_J": float(np.max(np.abs(J.data.astype(np.float64) - v)) / nJ),
                     "tolerance_J": 1e-5 if prec.startswith("fp32") else 1e-12}
        del R, J
    return out


def droplet_problem(size: int, precision: str, shape=None):
    """Droplet on its moving mesh (contact angle drawn from U[60, 120]
    degrees with seed 0) in a BDF2 step of dt = 1e-3: seeded velocities,
    pressures, multipliers and mesh displacements (a fraction of the element
    size), the hemisphere as both previous time levels."""
    from pyoomph_gb300 import ale
    rng = np.random.default_rng(0)
    theta = float(rng.uniform(60.0, 120.0))
    P = ale.DropletProblem(N=size, contact_angle_deg=theta, jacobian_precision=precision)
    if shape is not None:
        P.nthreads_cap, P.smem_budget = shape
    P.initialise()
    v0 = P._values0
    v = v0.copy()
    v[:, 2:] = rng.normal(0.0, 0.1, size=(v.shape[0], 4))
    v[:, 0:2] += rng.normal(0.0, 0.04 / size ** 2, size=(v.shape[0], 2))
    v[P.pinned] = v0[P.pinned]
    P.set_state(v, [v0, v0])
    w = ale.bdf_weights(2, 1e-3)
    P.set_params(__bdf0=w[0], __bdf1=w[1], __bdf2=w[2])
    return P, theta


def droplet_algorithmic_bytes(P) -> int:
    """Compulsory HBM bytes of one fused launch: connectivity, nodal values
    (current and two previous levels) and reference positions read once,
    element residuals and matrices written once."""
    jb = 8 if P._prec == "f64" else 4
    b = P.n_nodes * P.nval * 8 * 3 + P.n_nodes * 2 * 8
    for dc, conn in zip(P.domains, P.conns):
        b += conn.size * 4 + conn.shape[0] * (dc.nloc * 8 + dc.nloc * dc.nloc * jb)
    return int(b)


def run_droplet(args):
    """Moving-mesh droplet: the fused bulk + interface + contact-line
    assembly (one element launch) of a BDF2 Newton step."""
    import torch
    torch.cuda.set_device(0)
    hbm_peak, peak_kind = _peaks()
    res = {}
    tuned = {}
    for prec in ("fp64", "fp32", "df64"):
        shape = None
        if args.autotune:
            from pyoomph_gb300 import autotune as AT
            cands = [(128, 64 * 1024), (256, 100 * 1024), (256, 200 * 1024), (512, 200 * 1024)]
            shape, table = AT.tune(f"droplet-{args.size}-{prec}", lambda c: droplet_problem(args.size, prec, c)[0],
                                   cands, use_cache=False)
            tuned[prec] = {"threads_cap_smem_budget": shape, "ms_per_assembly": table}
        P, theta = droplet_problem(args.size, prec, shape)
        asm = lambda: P.assemble_device(with_jacobian=True)
        for _ in range(args.warmup):
            asm()
        torch.cuda.synchronize()
        with ClockSampler(0) as cs:
            ms = time_steps(torch, asm, args.steps, 0)
        P.check()
        P.set_stage_timing(True)
        for _ in range(max(3, min(args.steps, 10))):
            asm()
        stage_ms, calls = P.stage_times()
        P.set_stage_timing(False)
        stage_ms = stage_ms / max(calls, 1)
        xh = P.x_dev[:P.n_dof].cpu().pin_memory()
        Rh = torch.empty(P.n_dof, dtype=torch.float64).pin_memory()
        Jh = torch.empty(P.nnz, dtype=P.J_dev.dtype).pin_memory()

        def e2e():
            P.x_dev[:P.n_dof].copy_(xh, non_blocking=True)
            P.assemble_device(with_jacobian=True)
            Rh.copy_(P.R_dev[:P.n_dof], non_blocking=True)
            Jh.copy_(P.J_dev[:P.nnz], non_blocking=True)

        ms_e2e = time_steps(torch, e2e, max(3, args.steps), args.warmup)
        P.capture_assembly(with_jacobian=True)
        ms_graph = time_steps(torch, P.assemble_graph, args.steps, args.warmup)
        P.check()
        P.set_persistent(True)
        ms_persistent = time_steps(torch, asm, args.steps, args.warmup)
        P.set_persistent(False)
        P.check()
        res[prec] = dict(ms_persistent=ms_persistent, P=P, ms=ms, stage_ms=stage_ms, ms_e2e=ms_e2e, clocks=cs.summary(), ms_graph=ms_graph,
                         h2d=int(P.n_dof * 8), d2h=int(P.n_dof * 8 + P.nnz * P.J_dev.element_size()))
    peak64 = fp64_peak_tflops(torch)
    m = res["fp64"]
    P = m["P"]
    n_elem = P.n_elem
    elem_ms = float(m["stage_ms"][1])
    abytes = droplet_algorithmic_bytes(P)
    flops = sum(dc.flops * c.shape[0] for dc, c in zip(P.domains, P.conns))
    line = {
        "metric": "element residual+Jacobian assemblies/s (full CSR assembly)",
        "value": n_elem / (m["ms"] / 1e3), "unit": "elements/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": m["ms"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOADS["droplet"][0], "mesh_side": args.size, "n_elem": n_elem,
                   "n_elem_per_domain": {"bulk": int(P.conns[0].shape[0]), "interface": int(P.conns[1].shape[0]),
                                         "contact_line": 1},
                   "n_dof": P.n_dof, "nnz": P.nnz, "contact_angle_deg": theta, "dt": 1e-3, "ohnesorge": 0.1,
                   "jacobian": "fp64", "residual": "fp64",
                   "l2": "working set per step > L2 (element matrices + CSR + contribution lists)"},
        "stage_ms": {"dof_scatter": float(m["stage_ms"][0]), "element_kernel_fused": elem_ms,
                     "residual_gather": float(m["stage_ms"][2]), "jacobian_gather": float(m["stage_ms"][3])},
        "roofline": {"bound": "hbm", "kernel": P.kernel.name, "achieved": abytes / (elem_ms / 1e3) / 1e9,
                     "peak": hbm_peak, "unit": "GB/s", "frac": abytes / (elem_ms / 1e3) / 1e9 / hbm_peak,
                     "peak_kind": peak_kind, "algorithmic_bytes_per_launch": abytes,
                     "traffic": (measured_traffic(P.kernel.name, n_elem) or {}).get("bytes"),
                     "traffic_capture": measured_traffic(P.kernel.name, n_elem)},
        "compute_roofline": {"pipe": "fp64", "kernel": P.kernel.name, "flops_per_launch": flops,
                             "achieved": flops / (elem_ms / 1e3) / 1e12, "peak": peak64, "unit": "TFLOP/s",
                             "frac": flops / (elem_ms / 1e3) / 1e12 / peak64,
                             "peak_kind": "measured in this run: cuBLAS DGEMM 4096^3 (torch.matmul float64)",
                             "flops": "counted from the generated kernel's operation structure, FMA = 2"},
        "e2e": {"value": n_elem / (m["ms_e2e"] / 1e3), "unit": "elements/s", "h2d_bytes_per_step": m["h2d"],
                "d2h_bytes_per_step": m["d2h"], "ms_per_step": m["ms_e2e"]},
        "gpu_launches": P.launch_count(True) * args.steps,
        "clocks": m["clocks"],
        "cuda_graph": {"ms_per_step": m["ms_graph"], "value": n_elem / (m["ms_graph"] / 1e3), "launches_per_step": 1},
        "persistent_fused_launch_ms_per_step": {"fp64": m["ms_persistent"], "fp32": res["fp32"]["ms_persistent"]},
        "launch_shape": {"threads": P.kernel.threads, "smem_bytes": P.kernel.smem_bytes,
                         "elems_per_block": [dc.epb for dc in P.domains], "autotuned": tuned or None},
    }
    r32 = res["fp32"]
    P32 = r32["P"]
    k32 = float(r32["stage_ms"][1]) / 1e3
    f64_32 = sum(dc.flops * c.shape[0] for dc, c in zip(P32.domains, P32.conns))
    f32_32 = sum(dc.flops32 * c.shape[0] for dc, c in zip(P32.domains, P32.conns))
    line["fp32_jacobian"] = {"value": n_elem / (r32["ms"] / 1e3), "unit": "elements/s",
                             "ms_per_step": r32["ms"], "element_kernel_ms": k32 * 1e3,
                             "fp64_tflops": f64_32 / k32 / 1e12, "fp32_tflops": f32_32 / k32 / 1e12,
                             "fp64_frac_of_dgemm": f64_32 / k32 / 1e12 / peak64,
                             "e2e": {"value": n_elem / (r32["ms_e2e"] / 1e3),
                                     "h2d_bytes_per_step": r32["h2d"], "d2h_bytes_per_step": r32["d2h"]},
                             "cuda_graph_ms_per_step": r32["ms_graph"]}
    rdf = res["df64"]
    Pdf = rdf["P"]
    kdf = float(rdf["stage_ms"][1]) / 1e3
    f64_df = sum(dc.flops * c.shape[0] for dc, c in zip(Pdf.domains, Pdf.conns))
    fdf_df = sum(dc.flops_df64 * c.shape[0] for dc, c in zip(Pdf.domains, Pdf.conns))
    # full-size parity against the FP64 kernel on the same state
    Pdf.assemble_device(with_jacobian=True)
    P.assemble_device(with_jacobian=True)
    jdiff = float((Pdf.J_dev[:P.nnz] - P.J_dev[:P.nnz]).abs().max() / P.J_dev[:P.nnz].abs().max())
    rdiff = float((Pdf.R_dev[:P.n_dof] - P.R_dev[:P.n_dof]).abs().max() / P.R_dev[:P.n_dof].abs().max())
    line["df64_jacobian"] = {
        "what": "FP64 residual, geometry and coefficients; the Jacobian contraction in double-float "
                "(hi + lo pairs of FP32) on the FP32 pipes; FP64 Jacobian values",
        "value": n_elem / (rdf["ms"] / 1e3), "unit": "elements/s", "ms_per_step": rdf["ms"],
        "element_kernel_ms": kdf * 1e3, "kernel": Pdf.kernel.name,
        "fp64_tflops": f64_df / kdf / 1e12, "df64_contraction_tflops_fp64_equivalent": fdf_df / kdf / 1e12,
        "max_rel_jacobian_difference_vs_fp64": jdiff, "max_rel_residual_difference_vs_fp64": rdiff,
        "e2e": {"value": n_elem / (rdf["ms_e2e"] / 1e3), "unit": "elements/s",
                "h2d_bytes_per_step": rdf["h2d"], "d2h_bytes_per_step": rdf["d2h"], "ms_per_step": rdf["ms_e2e"]},
        "cuda_graph_ms_per_step": rdf["ms_graph"],
        "launch_shape": {"threads": Pdf.kernel.threads, "smem_bytes": Pdf.kernel.smem_bytes,
                         "elems_per_block": [dc.epb for dc in Pdf.domains]}}
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = droplet_cpu_baseline(args.size)
    print(json.dumps(line), flush=True)


def measure_droplet_compact(size: int, steps: int, warmup: int, hbm_peak: float, peak64: float):
    """The moving-mesh droplet's fused assembly (bulk + interface + contact
    line in one launch) per Jacobian precision, device-resident and end to
    end; df64's Jacobian against the FP64 one on the same state."""
    import torch
    out = {"workload": WORKLOADS["droplet"][0], "mesh_side": size}
    Ps = {}
    for prec in ("fp64", "fp32", "df64"):
        P, theta = droplet_problem(size, prec)
        asm = lambda: P.assemble_device(with_jacobian=True)
        ms = time_steps(torch, asm, steps, warmup)
        P.check()
        P.set_stage_timing(True)
        for _ in range(5):
            asm()
        st, calls = P.stage_times()
        P.set_stage_timing(False)
        st = st / max(calls, 1)
        xh = P.x_dev[:P.n_dof].cpu().pin_memory()
        Rh = torch.empty(P.n_dof, dtype=torch.float64).pin_memory()
        Jh = torch.empty(P.nnz, dtype=P.J_dev.dtype).pin_memory()

        def e2e():
            P.x_dev[:P.n_dof].copy_(xh, non_blocking=True)
            P.assemble_device(with_jacobian=True)
            Rh.copy_(P.R_dev[:P.n_dof], non_blocking=True)
            Jh.copy_(P.J_dev[:P.nnz], non_blocking=True)

        ms_e2e = time_steps(torch, e2e, steps, warmup)
        flops = sum(dc.flops * c.shape[0] for dc, c in zip(P.domains, P.conns))
        out[prec] = {"ms_per_step": ms, "value": P.n_elem / (ms / 1e3), "unit": "elements/s",
                     "element_kernel_fused_ms": float(st[1]), "kernel": P.kernel.name,
                     "e2e": {"value": P.n_elem / (ms_e2e / 1e3), "ms_per_step": ms_e2e,
                             "h2d_bytes_per_step": int(P.n_dof * 8),
                             "d2h_bytes_per_step": int(P.n_dof * 8 + P.nnz * P.J_dev.element_size())}}
        if prec == "fp64":
            out[prec]["fp64_frac_of_dgemm"] = flops / (float(st[1]) / 1e3) / 1e12 / peak64
        Ps[prec] = P
        out.update(n_elem=P.n_elem, n_dof=P.n_dof, nnz=P.nnz, contact_angle_deg=theta)
    Ps["fp64"].assemble_device(with_jacobian=True)
    Ps["df64"].assemble_device(with_jacobian=True)
    Jf, Jd = Ps["fp64"].J_dev[:Ps["fp64"].nnz], Ps["df64"].J_dev[:Ps["df64"].nnz]
    out["df64_max_rel_jacobian_difference_vs_fp64"] = float((Jd - Jf).abs().max() / Jf.abs().max())
    return out


def droplet_cpu_baseline(size: int, seconds: float = 10.0):
    """The ALE oracle (numpy, vectorised over elements, complex-step
    Jacobians) on one host core: element residuals and Jacobians of the
    three domains on a bounded mesh."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import ale_oracle as A
    side = min(size, 24)
    D = A.droplet(side)
    v = A.initial_values(D)
    p = {"dynamic_viscosity": 0.1, "surface_tension": 1.0, "contact_angle": 1.3,
         "__bdf0": 1500.0, "__bdf1": -2000.0, "__bdf2": 500.0}
    ne = D.tri.shape[0] + D.line.shape[0] + 1
    A.element_res_jac(D, v, [v, v], p)
    t0 = time.perf_counter()
    n = 0
    while time.perf_counter() - t0 < seconds:
        A.element_res_jac(D, v, [v, v], p)
        n += 1
    dt = time.perf_counter() - t0
    return {"value": ne * n / dt, "unit": "elements/s", "cores": 1, "kind": "port",
            "sample": f"droplet side {side} ({ne} elements), {n} element R+J evaluations in {dt:.1f}s "
                      f"(oracle/ale_oracle.py, numpy + complex step; no sparse assembly)"}


def run_reference(args):
    """The reference arm: the oracle's restated reference assembly (pyoomph's
    JIT flags) on every host core, one spawned process per core, each step
    at least one whole assembly of the bench's mesh per process."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    seconds = max(1.0, min(20.0, 60.0 / max(1, args.steps + args.warmup)))
    vals = []
    t_run = time.perf_counter()
    if args.workload == "droplet":
        for _ in range(args.warmup):
            droplet_cpu_baseline(args.size, seconds / 4)
        for _ in range(args.steps):
            cb = droplet_cpu_baseline(args.size, seconds)
            vals.append(cb["value"])
        side = min(args.size, 24)
    else:
        side = _sample_side(args.workload, args.size)
        pool = CpuPool(args.workload, side, threads)
        try:
            for _ in range(args.warmup):
                pool.measure(0.0)
            n_total = 0
            for _ in range(args.steps):
                v, n, flags = pool.measure(seconds)
                vals.append(v)
                n_total += n
        finally:
            pool.close()
        cb = {"unit": "elements/s", "cores": threads, "kind": "port", "mesh_side": side,
              "sample": _cpu_sample_text(args.workload, side, n_total, seconds * args.steps, flags, threads)}
    value = float(np.median(vals))
    cb["value"] = value
    wall = time.perf_counter() - t_run
    line = {"impl": "reference", "metric": "element residual+Jacobian assemblies/s (full CSR assembly)",
            "value": value, "unit": "elements/s", "n_gpus": int(os.environ.get("WORLD_SIZE", "1")),
            "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOADS[args.workload][0], "mesh_side": side, "jacobian": "fp64",
                       "residual": "fp64"},
            "wall_s": wall,
            "cpu_baseline": cb, "e2e": {"value": value, "unit": "elements/s", "h2d_bytes_per_step": 0,
                                        "d2h_bytes_per_step": 0}}
    if side != args.size:
        line["config"]["bench_mesh_side"] = args.size
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="ns", choices=list(WORKLOADS))
    ap.add_argument("--size", type=int, default=None)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extras", action="store_true",
                    help="default NS run: skip the other workloads' compact records")
    ap.add_argument("--autotune", action="store_true", help="time the element kernels' launch shapes first")
    ap.add_argument("--requests", type=int, default=200)
    ap.add_argument("--rates", default="10,20,50")
    ap.add_argument("--ns-side-max", type=int, default=None,
                    help="serving: cap the Navier-Stokes requests' sides (their solves stay on the host)")
    ap.add_argument("--device-solver", action="store_true",
                    help="serving: solve the Newton systems on the device (Poisson: batched BiCGStab; "
                         "Navier-Stokes from --ns-device-min-side: the saddle-point GMRES)")
    ap.add_argument("--ns-device-min-side", type=int, default=None,
                    help="serving: smallest Navier-Stokes side solved on the device (default: the server's)")
    args = ap.parse_args()
    if args.size is None:
        args.size = WORKLOADS[args.workload][1]
    if args.warmup < 3:
        args.warmup = 3
    if args.workload == "serving":
        run_serving(args)
    elif args.workload == "droplet" and args.impl != "reference":
        run_droplet(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()
