"""Benchmark of the Mallard residual-and-update path on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--n 1024]
                    [--form fp32_learned] [--forms fp64,fp64_fast,fp32]

Workload (the 2D four-quadrant Riemann configuration): cartesian_tri mesh of
n x n quads split into 2 n^2 triangles (n = 1024 -> 2,097,152 cells) on the
unit square, relabelled by a seeded random cell permutation (seed 20261203)
and reverse-Cuthill-McKee ordered inside the library; TENO p = 3 (legendre),
HLLC, SSPRK3 with CFL 0.5, extrapolation (transmissive) boundaries, gamma
1.4, quadrant states split at x = y = 0.8.  Synthetic, seeded data.  The
TENO weighting is the robust variant (the corrected cut-off weighting with
first-order boundary cells, a range scaling and a positivity fallback per
cell, and a guarded HLLC star pressure): it runs this state to t = 0.3,
which the reference's weighting (non-finite within one step) and the
corrected one (within ~15 steps) do not.

Forms (all on the GPU, same mesh, state and steps):
  fp64          the plain path, FP64 with the reference's operation order
  fp64_fast     FP64 with FMA contraction
  fp32          reconstruction and flux in FP32, state and accumulation FP64
  fp32_learned  fp32 + the learned stencil selector (the headline by default)
The headline line carries the headline form's rate, and "forms" every
form's rate, per-kernel times and its density L1 / L-infinity and mass /
energy differences against the plain FP64 state after the same steps.  A
timed state that is not finite, or a non-zero status word, prints a
"status" line without a value and exits 1.

One step = spectral radius + dt + three stages of (reconstruction, face flux,
residual gather + update), plus one selector inference every fourth step in
the learned form (--sel-interval), all on the GPU, replayed as CUDA graphs.
Inputs (tables 3.4-7 KB per cell, 7-15 GB) are far larger than L2, so no
explicit flush is done.

Metric: Mcell-updates/s = cells x steps / seconds / 1e6 (one cell-update =
one cell advanced one full SSPRK3 step).

Further sections of the line: "end_time" runs the four-quadrant problem to
t = 0.3 (the learned form at the headline size; the plain FP64 path and the
learned form at --end-time-n, with the error between them); "c5" times the
learned form against the plain FP64 path on 2048^2 (8.4M cells); "wedge"
times the 4M-cell supersonic wedge (Delaunay ramp channel, viscous at Re 1e5
with no-slip walls), plain FP64 against FP32 + learned selector; "batched"
runs the ensemble workload (256 four-quadrant cases of uneven mesh size) to
its 500 steps with the batched FP32 form.

--impl reference times the CPU oracle (the restatement of the reference's
algorithm, FP64, all host threads) on the same 1024^2 mesh, built by the
oracle's own mesh generator and cell permutation (the GPU library is not
loaded in that process).
"""

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "tests"))

METRIC = "Mcell-updates/s on 1 GB300: FP64 plain vs FP32+learned TENO at matched L1 error"
UNIT = "Mcell-updates/s"
SEED = 20261203
CFL = 0.5
T_END = 0.3
CPU_SAMPLE_N = 256
SEL_THRESHOLD = 0.995
WEDGE_CFL = 0.4
GAS = dict(gamma=1.4, p_ref=101325.0, T_ref=298.15, rho_ref=1.225)
# the four-quadrant states (rho, u, v, p) of UR, UL, LL, LR
QUADRANTS = ((1.5, 0.0, 0.0, 1.5),
             (0.532258064516129, 1.206045378311055, 0.0, 0.3),
             (0.137992831541219, 1.206045378311055, 1.206045378311055, 0.029032258064516),
             (0.532258064516129, 0.0, 1.206045378311055, 0.3))


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=8)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=1024, help="quads per side (cells = 2 n^2)")
    ap.add_argument("--variant", default="robust", choices=["reference", "corrected", "robust"])
    ap.add_argument("--form", default="fp32_learned", choices=["fp64", "fp64_fast", "fp32", "fp32_learned"],
                    help="headline form: fp64 = the reference's rounding (bit-faithful); fp64_fast = FMA-contracted "
                         "FP64; fp32 = FP32-bulk reconstruction and flux; fp32_learned = fp32 + learned selector")
    ap.add_argument("--forms", default="fp64,fp64_fast,fp32",
                    help="other forms timed on the same workload (comma list, '' for none); fp64 is also the "
                         "error reference")
    ap.add_argument("--end-time-n", type=int, default=256,
                    help="mesh size of the end-time accuracy run (plain FP64 and learned form to t = 0.3); 0 skips "
                         "the end-time section")
    ap.add_argument("--c5-n", type=int, default=2048, help="mesh size of the c5 section (0 skips it)")
    ap.add_argument("--wedge-n", type=int, default=816,
                    help="rows of the ramp-channel lattice (3n+1 columns; 816 -> 4.0M triangles); 0 skips it")
    ap.add_argument("--wedge-develop", type=int, default=300,
                    help="untimed steps of the wedge from its uniform start before the timed ones")
    ap.add_argument("--wedge-total", type=int, default=0,
                    help="total steps of the wedge (the configuration's 2000); the development steps become "
                         "total - warmup - steps (0: --wedge-develop)")
    ap.add_argument("--wedge-re", type=float, default=1e5,
                    help="Reynolds number of the wedge on the ramp length (viscous flux, no-slip walls); 0 = inviscid")
    ap.add_argument("--wedge-variant", default="robust", choices=["corrected", "robust"],
                    help="TENO variant of the wedge (the corrected one keeps high order in the wall cells but goes "
                         "non-finite at the ramp wall before the configured 2000 steps)")
    ap.add_argument("--batch-cases", type=int, default=256,
                    help="cases of the batched section (the four-quadrant ensemble); 0 skips it")
    ap.add_argument("--batch-steps", type=int, default=500, help="total steps of the batched section")
    ap.add_argument("--sel-interval", type=int, default=4,
                    help="steps per selector prediction in the learned form (1 = every step; at CFL 0.5 a wave "
                         "crosses about 0.12 of a cell per step, so 4 steps stay inside the neighbour check's "
                         "one-cell margin)")
    ap.add_argument("--shape", type=int, default=-1,
                    help="fix the FP32 reconstruction's launch shape (0-7) instead of autotuning it")
    ap.add_argument("--cpu-sample-n", type=int, default=CPU_SAMPLE_N)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    return ap.parse_args()


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("LOCAL_RANK", 0)), int(os.environ.get("WORLD_SIZE", 1))


def four_quadrant_state(cell_coords, split=0.8):
    """Conservatives and primitives of the four-quadrant state per cell, as
    the reference's analytical initialisation computes them
    (src/solver/solver_initialize.cpp:159-185, physics.cpp:69-73)."""
    x, y = cell_coords[:, 0], cell_coords[:, 1]
    right, top = x >= split, y >= split
    prim = np.zeros((len(x), 4))
    for sel, st in zip((right & top, ~right & top, ~right & ~top, right & ~top), QUADRANTS):
        prim[sel] = st
    g = GAS["gamma"]
    R = GAS["p_ref"] / (GAS["T_ref"] * GAS["rho_ref"])
    cp = R * g / (g - 1.0)
    cv = cp / g
    rho, u, v, p = prim.T
    T = p / (rho * R)
    e = cv * T
    E = e + 0.5 * (u * u + v * v)
    h = e + p / rho
    return (np.ascontiguousarray(np.stack([rho, rho * u, rho * v, rho * E], 1)),
            np.ascontiguousarray(np.stack([u, v, p, T, h], 1)))


def case_mesh(n):
    import mallard_gb300 as mg
    m = mg.Mesh.generate("cartesian_tri", n, n, 1.0, 1.0)
    m.permute_cells(SEED)
    return m


def workload_config(args, n):
    return {"workload": f"four-quadrant Riemann, cartesian_tri {n}x{n} quads -> {2 * n * n} triangles, "
                        f"seeded permutation + RCM, TENO p3 legendre + HLLC, SSPRK3 CFL {CFL}, transmissive BCs",
            "cells": 2 * n * n, "teno_variant": args.variant, "seed": SEED,
            "l2": "inputs larger than L2 (TENO tables 3.4-7 KB/cell); no flush", "parallelism": "replicas"}


# ---------------------------------------------------------------------------
# clocks during the timed region
# ---------------------------------------------------------------------------

class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (FileNotFoundError, OSError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.t.join(timeout=2)
        sm, smax, reasons, power = [], [], set(), []
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
                power.append(float(parts[3]))
            except ValueError:
                continue
            for name, val in zip(names, parts[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm), "power_w_max": max(power) if power else None}


# ---------------------------------------------------------------------------
# CPU oracle legs (no GPU library in these: the oracle's own mesh generator
# and cell permutation build the same mesh)
# ---------------------------------------------------------------------------

def oracle_case(n, variant, threads):
    from oracle import Oracle, OracleCase, OracleMesh
    Oracle().set_threads(threads)
    om = OracleMesh.generate("cartesian_tri", n, n, 1.0, 1.0)
    om.permute_cells(SEED)
    oc = OracleCase(om, recon="TENO", basis="legendre", poly_order=3, riemann="HLLC", **GAS)
    oc.set_teno_variant({"reference": 0, "corrected": 1, "robust": 2}[variant])
    for z in range(1, 5):
        oc.add_boundary(z, "extrapolation")
    U, W = four_quadrant_state(om.cell_coords)
    oc.set_state(U, W)
    return oc, om.n_cells


def cpu_oracle_rate(n, steps, warmup, variant):
    """Cell-updates/s of the oracle on the n x n workload, all host threads:
    W untimed then K timed consecutive steps from the initial state."""
    threads = max(1, os.cpu_count() or 1)
    t0 = time.perf_counter()
    oc, cells = oracle_case(n, variant, threads)
    setup = time.perf_counter() - t0
    if warmup:
        oc.run(CFL, warmup)
    t0 = time.perf_counter()
    oc.run(CFL, steps)
    secs = time.perf_counter() - t0
    U, _ = oc.get_state()
    return cells * steps / secs / 1e6, threads, secs, cells, setup, bool(np.isfinite(U).all())


def run_reference(args):
    rank, _, world = dist_env()
    if rank != 0:
        return
    rate, threads, secs, cells, setup, finite = cpu_oracle_rate(args.n, args.steps, args.warmup, args.variant)
    sample = (f"the full workload: cartesian_tri {args.n}x{args.n} ({cells} cells), {args.steps} timed steps after "
              f"{args.warmup} warm-up, {threads} OpenMP threads (setup {setup:.1f} s untimed)")
    line = {"impl": "reference", "metric": METRIC, "value": rate, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": secs * 1e3 / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": workload_config(args, args.n),
            "reference_path": "CPU oracle (oracle/mallard_oracle.cpp: the reference's algorithm restated, FP64, "
                              "OpenMP with atomic scatter like Kokkos::OpenMP); the reference itself does not build "
                              "here (its Kokkos, KokkosKernels and toml11 submodules are empty)",
            "finite": finite,
            "cpu_baseline": {"value": rate, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": rate, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# GPU leg
# ---------------------------------------------------------------------------

def teno_flops_per_cell(precision, K=10, M=20, nq=2, stencils=4):
    """FP64 flops of one TENO reconstruction per cell (4 variables), central
    branch, counting a fused multiply-add as 2 and a divide as 1:
    per stencil b (2 per neighbour), P b (2 K' M'), the smoothness
    indicator (full K'^2 + K' products in the exact form, the symmetric
    half in the fast form), x^6 and 1/x; then 3 faces x nq points x K'
    shape terms (3 ops exact, 2 fast)."""
    KR, MR = K - 1, M - 1
    if precision == "fp64":
        si, pw, face = 2 * KR * KR + 2 * KR, 12 + 1, 3
    else:
        si, pw, face = 2 * (KR * (KR + 1) // 2) + 2 * KR, 3 + 1, 2
    per_var = stencils * (2 * MR + 2 * KR * MR + si + pw) + 3 * nq * KR * face + 10
    return 4 * per_var


def load_selector(device):
    """The trained selector weights shipped with the package; trains a quick
    one on the GPU when they are missing."""
    from mallard_gb300.selector import Selector, default_weights_path
    path = default_weights_path()
    if path.exists():
        sel = Selector(device=device)
        sel.load(path)
        return sel, str(path.relative_to(ROOT))
    from mallard_gb300.train_selector import train
    sel, _ = train(None, quick=True, log=lambda *a: print(*a, file=sys.stderr))
    return sel, "trained at startup (quick)"


def selector_summary(selector, stats, interval=1):
    when = "once per step" if interval == 1 else f"every {interval} steps"
    return {"weights": selector[1], "central_threshold": SEL_THRESHOLD,
            "directional_predictions": "not trusted (full TENO)",
            "predict": f"{when}, from the step's initial state; trusted where the face neighbours are confident too",
            "confident_cells": stats["confident_cells"] / stats["cells"],
            "confident_variables": stats["confident_variables"] / (4 * stats["cells"]),
            "stencils_evaluated_frac": stats["stencils_evaluated"] / stats["stencils_full"],
            "error_flag": stats["error"]}


FORMS = {
    # form: (precision, learned selector)
    "fp64": ("fp64", False),
    "fp64_fast": ("fp64_fast", False),
    "fp32": ("fp32", False),
    "fp32_learned": ("fp32", True),
}


def make_solver(m, args, form, device, selector):
    import mallard_gb300 as mg
    prec, learned = FORMS[form]
    s = mg.Solver(m, face_reconstruction="TENO", basis_type="legendre", basis_order=3, riemann_solver="HLLC",
                  boundaries=[{"name": z, "type": "extrapolation"} for z in ("right", "top", "left", "bottom")],
                  teno_variant=args.variant, reorder=True, device=device, precision=prec, **GAS)
    if learned:
        s.attach_selector(selector[0], threshold=SEL_THRESHOLD, interval=args.sel_interval)
    return s


def errors_vs(m, U, U_ref):
    vol = m.cell_volume
    fin = bool(np.isfinite(U).all() and np.isfinite(U_ref).all())
    if not fin:
        return {"finite": False, "density_l1_rel_err": None, "density_linf_rel_err": None}
    d = np.abs(U[:, 0] - U_ref[:, 0])
    i = int(np.argmax(d))
    return {"density_l1_rel_err": float(np.sum(vol * d) / np.sum(vol * np.abs(U_ref[:, 0]))),
            "density_linf_rel_err": float(d.max() / np.abs(U_ref[:, 0]).max()),
            "density_linf_at": [round(float(x), 4) for x in m.cell_coords[i]],
            "mass_rel_diff": float(abs(np.sum(vol * U[:, 0]) - np.sum(vol * U_ref[:, 0])) / np.sum(vol * U_ref[:, 0])),
            "energy_rel_diff": float(abs(np.sum(vol * U[:, 3]) - np.sum(vol * U_ref[:, 3])) /
                                     np.sum(vol * U_ref[:, 3]))}


def autotune(s, args, U0, W0):
    if args.shape >= 0:
        s.set_launch_shape(args.shape)
        return {"chosen_shape": args.shape, "ms_per_shape": None, "shapes": "fixed by --shape"}
    shape, tms = s.autotune()
    s.set_state(U0, W0)
    return {"chosen_shape": shape, "ms_per_shape": [round(x, 4) for x in tms],
            "shapes": "0: 128 thr/<=128 regs, 1: 128/<=80, 2: 128/<=64, 3: 256/<=64, "
                      "4-7: staged (bulk copies to shared memory, 1 stencil slot per warp) 4 warps/<=80, "
                      "2 warps/<=72, 1 warp/<=72, 4 warps/<=72"}


def time_form(m, args, form, U0, W0, device, selector, barrier=None, clocks=None):
    """One form on the workload: device-timed rate over K graph-replayed steps
    after W warm-up steps (CUDA events on the solver's stream), the final
    state, per-kernel times from a second pass with events around every
    launch, and the selector's statistics."""
    import torch
    s = make_solver(m, args, form, device, selector)
    stream = torch.cuda.Stream()
    s.set_stream(stream.cuda_stream)
    s.set_state(U0, W0)
    tune = autotune(s, args, U0, W0) if FORMS[form][0] == "fp32" else None
    s.launch(CFL, args.warmup)
    s.synchronize()
    if clocks:
        clocks.start()
        time.sleep(0.3)
    if barrier:
        barrier()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    s.launch(CFL, args.steps)
    e1.record(stream)
    e1.synchronize()
    if barrier:
        barrier()
    ms = e0.elapsed_time(e1)
    clk = clocks.stop() if clocks else None
    flags = s.status()
    U, _ = s.get_state()
    stats = s.selector_stats() if FORMS[form][1] else None
    s.set_state(U0, W0)
    s.launch(CFL, args.warmup)
    s.kernel_timing(True)
    s.launch(CFL, args.steps)
    kt = s.kernel_times()
    s.kernel_timing(False)
    return s, {"ms": ms, "U": U, "flags": flags, "stats": stats, "kt": kt, "clocks": clk, "tune": tune}


def kernel_bytes(kind, precision, learned, cells, faces, solver, stats):
    """Algorithmic (compulsory) bytes of one launch of a kernel class:
    recon: the library's traffic model (tables of the stencils evaluated,
    shapes, face slots, the state gathered once per cell, face states
    written); flux: per flux face the face states of both sides, the flux x
    area written and the face geometry; update: per cell the gather list,
    1/volume and the state rows one SSPRK3 stage reads and writes (averaged
    over the three), plus every face's flux once; cfl: per cell its faces,
    its state row and the radius, per face its cells, normal and 1/distance;
    selector: neighbour ids of all stencils, the state gathered once per
    cell, predictions, the weight image once."""
    fp32 = precision == "fp32"
    fw = 4 if fp32 else 8
    if kind == "recon":
        full, _ = solver.traffic_model()
        if learned and stats:
            per_stencil = 19 * (4 + 4 * 9)
            return stats["stencils_evaluated"] * per_stencil + full - stats["stencils_full"] * per_stencil + cells * 4
        return full
    if kind == "flux":
        return faces * (2 * 2 * 4 * fw + 32 + 8 + 16 + 8 + 1)
    if kind == "update":
        rows = (96 + 160 + 64) / 3.0 + (16 if fp32 else 16.0)
        return cells * (16 + 8 + rows) + faces * 32
    if kind == "cfl":
        return cells * (16 + (16 if fp32 else 32 + 48) + 8) + faces * (8 + 16 + 8)
    if kind == "selector" and stats:
        return stats["stencils_full"] * 19 * 4 + cells * (32 + 4) + 25216
    return 0


def run_to_time(s, t_end, chunk=50):
    """Steps s to exactly t_end: CFL steps (in chunks while far from it), and
    a last step shortened to end on t_end.  Returns (steps, wall seconds,
    status ok)."""
    t, steps = 0.0, 0
    t0 = time.perf_counter()
    while t < t_end and s.status() == 0:
        if t_end - t > 0.02:
            t += s.run(CFL, chunk)
            steps += chunk
            continue
        dt, _ = s.calc_dt(CFL)
        if t + dt >= t_end:
            s.take_step(t_end - t)
            t = t_end
        else:
            s.take_step(dt)
            t += dt
        steps += 1
    s.synchronize()
    return steps, time.perf_counter() - t0, s.status() == 0


def run_end_time(args, device, selector):
    """The four-quadrant problem to its end time t = 0.3: the learned form on
    the headline mesh (finite, steps, wall time), and at --end-time-n the
    plain FP64 path, the FP64-fast form, the FP32 form and the learned form,
    each stepped at its own CFL time step to exactly t = 0.3, with the
    others' errors against the FP64 state."""
    out = {"t_end": T_END}
    m = case_mesh(args.n)
    U0, W0 = four_quadrant_state(m.cell_coords)
    s = make_solver(m, args, "fp32_learned", device, selector)
    s.set_state(U0, W0)
    s.autotune()
    s.set_state(U0, W0)
    steps, wall, ok = run_to_time(s, T_END)
    U, _ = s.get_state()
    vol = m.cell_volume
    out[f"{args.n}x{args.n}"] = {"form": "fp32_learned", "steps": steps, "wall_s": wall,
                                 "finite": bool(np.isfinite(U).all()) and ok,
                                 "density_min": float(U[:, 0].min()), "density_max": float(U[:, 0].max()),
                                 "mass": float(np.sum(vol * U[:, 0]))}
    s.close()
    n = args.end_time_n
    if n > 0:
        m = case_mesh(n)
        U0, W0 = four_quadrant_state(m.cell_coords)
        finals, rec = {}, {}
        for form in ("fp64", "fp64_fast", "fp32", "fp32_learned"):
            s = make_solver(m, args, form, device, selector)
            s.set_state(U0, W0)
            steps, wall, ok = run_to_time(s, T_END)
            finals[form] = s.get_state()[0]
            rec[form] = {"steps": steps, "wall_s": wall, "finite": bool(np.isfinite(finals[form]).all()) and ok}
            if form == "fp32_learned":
                rec[form]["selector"] = selector_summary(selector, s.selector_stats(), args.sel_interval)
            s.close()
        # fp64_fast (the same scheme with FMA contraction, ~1e-16 per operation)
        # is the control: how far a perturbation at round-off grows by t_end
        for form in ("fp64_fast", "fp32", "fp32_learned"):
            rec[form].update(errors_vs(m, finals[form], finals["fp64"]))
        out[f"{n}x{n}_vs_fp64"] = rec
    return out


def run_c5(args, device, selector):
    """The learned form against the plain FP64 path on the 2048^2
    four-quadrant mesh (8,388,608 cells): W + K steps each, rates and the
    density error after the same steps."""
    import torch
    n = args.c5_n
    m = case_mesh(n)
    U0, W0 = four_quadrant_state(m.cell_coords)
    out = {"workload": f"four-quadrant Riemann, cartesian_tri {n}x{n} -> {m.n_cells} triangles, seeded permutation "
                       f"+ RCM, TENO p3 ({args.variant}) + HLLC, CFL {CFL}", "cells": m.n_cells}
    finals = {}
    for form in ("fp64", "fp32_learned"):
        s = make_solver(m, args, form, device, selector)
        stream = torch.cuda.Stream()
        s.set_stream(stream.cuda_stream)
        s.set_state(U0, W0)
        if form == "fp32_learned":
            s.autotune()
            s.set_state(U0, W0)
        s.launch(CFL, args.warmup)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        s.launch(CFL, args.steps)
        e1.record(stream)
        e1.synchronize()
        ms = e0.elapsed_time(e1)
        finals[form] = s.get_state()[0]
        out[form] = {"value": m.n_cells * args.steps / (ms * 1e-3) / 1e6, "ms_per_step": ms / args.steps,
                     "finite": bool(np.isfinite(finals[form]).all()) and s.status() == 0}
        if form == "fp32_learned":
            out[form]["selector"] = selector_summary(selector, s.selector_stats(), args.sel_interval)
        s.close()
    out["fp32_learned"].update(errors_vs(m, finals["fp32_learned"], finals["fp64"]))
    out["speedup_learned_vs_fp64"] = out["fp32_learned"]["value"] / out["fp64"]["value"]
    return out


def run_wedge(args, device, selector):
    """The supersonic ramp channel (15 degree ramp at x = 0.5 in a 3 x 1
    channel, jittered-lattice Delaunay mesh of 2 nx ny triangles, Mach 2.5
    upt inflow, p_out outflow, TENO + Rusanov, CFL 0.4; viscous with no-slip
    walls at Re = --wedge-re, else slip walls): plain FP64 against FP32 +
    learned selector.  Each form first develops the flow from the uniform
    start for --wedge-develop steps (untimed: the early steps are mostly
    uniform flow, which flatters the selector), then runs W warm-up and K
    timed steps; the learned form's density error is taken against the
    plain one after all of them."""
    import torch

    import mallard_gb300 as mg
    from mallard_gb300.train_selector import wedge_setup
    develop = max(0, args.wedge_total - args.warmup - args.steps) if args.wedge_total > 0 else args.wedge_develop
    ny = args.wedge_n
    nx = 3 * ny + 1
    t0 = time.perf_counter()
    mesh = mg.Mesh.ramp_channel(nx, ny, 3.0, 1.0, 0.5, 15.0, 0.2, seed=SEED)
    re = args.wedge_re if args.wedge_re > 0 else None
    flow = (f"viscous Re {re:g} on the ramp length, Pr 0.72, Sutherland, no-slip adiabatic walls, cell gradients "
            f"of the reconstructed polynomials" if re else "inviscid (slip walls)")
    out = {"workload": f"ramp channel {nx}x{ny} lattice -> {mesh.n_cells} Delaunay triangles, 15 deg ramp, "
                       f"Mach 2.5, TENO p3 ({args.wedge_variant}) + Rusanov, SSPRK3 CFL {WEDGE_CFL}, {flow}; timed "
                       f"after {develop} development steps",
           "cells": mesh.n_cells, "mesh_s": time.perf_counter() - t0, "develop_steps": develop,
           "total_steps": develop + args.warmup + args.steps}
    finals = {}
    for form, prec in (("fp64", "fp64"), ("fp32_learned", "fp32")):
        t1 = time.perf_counter()
        s, U0, W0 = wedge_setup(mesh, precision=prec, reynolds=re, teno_variant=args.wedge_variant)
        if form == "fp32_learned":
            s.attach_selector(selector[0], threshold=SEL_THRESHOLD, interval=args.sel_interval)
        setup = time.perf_counter() - t1
        stream = torch.cuda.Stream()
        s.set_stream(stream.cuda_stream)
        s.set_state(U0, W0)
        if develop > 0:
            s.launch(WEDGE_CFL, develop)
            s.synchronize()
        if prec == "fp32":
            Ud, Wd = s.get_state()
            s.autotune()
            s.set_state(Ud, Wd)
        s.launch(WEDGE_CFL, args.warmup)
        s.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        s.launch(WEDGE_CFL, args.steps)
        e1.record(stream)
        e1.synchronize()
        ms = e0.elapsed_time(e1)
        U, _ = s.get_state()
        finals[form] = U
        out[form] = {"value": mesh.n_cells * args.steps / (ms * 1e-3) / 1e6, "ms_per_step": ms / args.steps,
                     "finite": bool(np.isfinite(U).all()) and s.status() == 0, "setup_s": setup}
        if form == "fp32_learned":
            out[form]["selector"] = selector_summary(selector, s.selector_stats(), args.sel_interval)
        s.close()
    out["fp32_learned"].update(errors_vs(mesh, finals["fp32_learned"], finals["fp64"]))
    out["speedup_learned_vs_fp64"] = out["fp32_learned"]["value"] / out["fp64"]["value"]
    return out


def run_batched(args, device):
    """The ensemble workload: n_cases independent four-quadrant problems on unit
    squares, mesh size drawn per case from {64, 128, 256, 512}^2 quads
    (cartesian_tri, so twice as many triangles), quadrant states drawn per
    case (rho ~ U[0.1, 2], p ~ U[0.03, 2], u, v ~ U[-1.5, 1.5]); the
    batched FP32 form with one launch per kernel over all cases, autotuned.
    W warm-up and K timed steps, then the rest of --batch-steps untimed;
    finite_cases counts the cases finite after all of them."""
    import torch

    import mallard_gb300 as mg
    from mallard_gb300.batch import Batch
    r = np.random.default_rng(SEED)
    sizes = [64, 128, 256, 512]
    draw = r.integers(0, 4, args.batch_cases)
    counts = [int((draw == i).sum()) for i in range(4)]
    used = [i for i in range(4) if counts[i]]
    t0 = time.perf_counter()
    meshes = [mg.Mesh.generate("cartesian_tri", sizes[i], sizes[i], 1.0, 1.0) for i in used]
    b = Batch(meshes, [counts[i] for i in used],
              boundaries=[{"name": z, "type": "extrapolation"} for z in ("right", "top", "left", "bottom")],
              riemann_solver="HLLC", teno_variant=args.variant, **GAS)
    cells = 0
    for g, i in enumerate(used):
        m = meshes[g]
        x, y = m.cell_coords[:, 0], m.cell_coords[:, 1]
        for k in range(counts[i]):
            q = np.column_stack([r.uniform(0.1, 2.0, 4), r.uniform(-1.5, 1.5, 4), r.uniform(-1.5, 1.5, 4),
                                 r.uniform(0.03, 2.0, 4)])
            sx, sy = r.uniform(0.3, 0.7, 2)
            quad = np.where(x >= sx, np.where(y >= sy, 0, 3), np.where(y >= sy, 1, 2))
            pr = q[quad]
            U, W = mg.state_from_primitives(pr[:, 0], pr[:, 1], pr[:, 2], pr[:, 3], **GAS)
            b.set_state(g, k, U, W)
            cells += m.n_cells
    setup = time.perf_counter() - t0
    shape, bps, ms = b.autotune()
    # autotuning ran reconstructions only; the states are unchanged
    stream = torch.cuda.Stream()
    b.set_stream(stream.cuda_stream)
    b.run(CFL, args.warmup)
    b.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    b.run(CFL, args.steps)
    e1.record(stream)
    e1.synchronize()
    secs = e0.elapsed_time(e1) * 1e-3
    flags_timed, _ = b.status()
    rest = max(0, args.batch_steps - args.warmup - args.steps)
    t1 = time.perf_counter()
    if rest:
        b.run(CFL, rest)
        b.synchronize()
    rest_s = time.perf_counter() - t1
    flags, times = b.status()
    b.close()
    case_cells = np.concatenate([np.full(counts[i], meshes[g].n_cells) for g, i in enumerate(used)])
    live = int(case_cells[flags_timed == 0].sum())
    return {"workload": f"{args.batch_cases} four-quadrant cases, cartesian_tri sizes {{64,128,256,512}}^2 quads "
                        f"drawn per case (seed {SEED}), random quadrant states, TENO p3 ({args.variant}) + HLLC, "
                        f"SSPRK3 CFL {CFL}, FP32 form, one launch per kernel over all cases",
            "cases_per_size": {f"{sizes[i]}x{sizes[i]}": counts[i] for i in range(4)}, "cells": cells,
            "value": live * args.steps / secs / 1e6, "unit": UNIT, "ms_per_step": secs * 1e3 / args.steps,
            "value_counts": "cells of the cases finite after the timed steps", "live_cells": live,
            "timing": "CUDA events on the batch's stream around the graph replays",
            "autotune": {"shape": shape, "ctas_per_sm": bps, "ms": np.round(ms, 4).tolist()},
            "total_steps": args.warmup + args.steps + rest, "rest_wall_s": rest_s,
            "finite_cases": int((flags == 0).sum()), "case_time_min": float(times.min()),
            "case_time_max": float(times.max()), "setup_s": setup}


def run_ours(args):
    import torch  # noqa: F401

    import mallard_gb300 as mg
    from mallard_gb300.replicas import Replicas

    reps = Replicas("nccl")
    rank, local, world = reps.rank, reps.local, reps.world
    barrier, max_over_ranks = reps.barrier, reps.max

    t_setup = time.perf_counter()
    m = case_mesh(args.n)
    U0, W0 = four_quadrant_state(m.cell_coords)
    cells = m.n_cells
    faces = int(m.zone_offsets[-1])
    head = args.form
    need_sel = FORMS[head][1] or "fp32_learned" in args.forms.split(",") or args.end_time_n or args.c5_n
    selector = load_selector(local) if need_sel else None
    setup_s = time.perf_counter() - t_setup

    # ---- the other forms (the plain FP64 path's final state is the error reference)
    forms, finals = {}, {}
    for form in [f for f in args.forms.split(",") if f and f != head]:
        s, r = time_form(m, args, form, U0, W0, local, selector)
        s.close()
        finals[form] = r["U"]
        kt = r["kt"]
        forms[form] = {"value": cells * args.steps / (r["ms"] * 1e-3) / 1e6, "ms_per_step": r["ms"] / args.steps,
                       "finite": bool(np.isfinite(r["U"]).all()) and r["flags"] == 0,
                       "kernel_ms_per_launch": {k: v[0] / max(v[1], 1) for k, v in kt.items() if v[1]}}
        if r["stats"]:
            forms[form]["selector"] = selector_summary(selector, r["stats"], args.sel_interval)
        if r["tune"]:
            forms[form]["autotune"] = r["tune"]
    # ---- the headline form
    clocks = ClockSampler(local)
    solver, r = time_form(m, args, head, U0, W0, local, selector, barrier=barrier, clocks=clocks)
    ms_max = max_over_ranks(r["ms"])
    value = cells * args.steps * world / (ms_max * 1e-3) / 1e6
    Uend, flags, kt, clk, stats = r["U"], r["flags"], r["kt"], r["clocks"], r["stats"]
    finite = bool(np.isfinite(Uend).all()) and flags == 0
    finals[head] = Uend
    if not finite:
        if rank == 0:
            print(json.dumps({"metric": METRIC, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                              "warmup": args.warmup, "status": "invalid: the timed state is not finite "
                                                               f"(status flags {flags}); no value is reported",
                              "config": workload_config(args, args.n)}), flush=True)
        reps.close()
        sys.exit(1)

    # ---- end to end through the public API with host buffers: each step
    # uploads the conserved state from pinned memory (the primitives are
    # recovered on the device), advances one CFL step and reads the new
    # conserved state back
    Uh = torch.empty((cells, 4), dtype=torch.float64, pin_memory=True).numpy()
    Uh[:] = U0
    barrier()
    e0 = time.perf_counter()
    for _ in range(args.steps):
        solver.set_state(Uh)
        solver.launch(CFL, 1)
        solver.synchronize()
        solver.get_state(Uh, primitives=False)
    e_secs = max_over_ranks(time.perf_counter() - e0)
    e2e_value = cells * args.steps * world / e_secs / 1e6
    h2d = cells * 4 * 8
    d2h = cells * 4 * 8

    # ---- roofline of the dominant kernel
    _, stage_bytes = solver.traffic_model()
    peaks = {}
    pk = ROOT / "MEASURED_PEAKS.json"
    if pk.exists():
        peaks = json.loads(pk.read_text())
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    total_ms = sum(x[0] for x in kt.values())
    kshare = {k: {"ms_per_launch": v[0] / max(v[1], 1), "launches": v[1], "share": v[0] / max(total_ms, 1e-30)}
              for k, v in kt.items() if v[1]}
    dom = max(kshare, key=lambda k: kshare[k]["share"])
    learned = FORMS[head][1]
    prec = FORMS[head][0]
    staged = bool(r["tune"]) and r["tune"]["chosen_shape"] >= 4
    fp32_name = "teno32_staged_kernel" if staged else "teno32_kernel"
    kernel_names = {"recon": (f"{fp32_name}<10,20,2,SEL>" if learned else
                              (f"{fp32_name}<10,20,2>" if prec == "fp32" else "teno_kernel<10,20,2>")),
                    "selector": "mlp_kernel<1> (tcgen05)", "flux": "flux32_kernel" if prec == "fp32" else "flux_kernel",
                    "update": "update_kernel", "cfl": "spectral_kernel"}
    for k in kshare:
        kshare[k]["algorithmic_bytes_per_launch"] = kernel_bytes(k, prec, learned, cells, faces, solver, stats)
        kshare[k]["achieved_gbs"] = kshare[k]["algorithmic_bytes_per_launch"] / (kshare[k]["ms_per_launch"] * 1e-3) / 1e9
    if "selector" in kshare:
        # a prediction is two launches (mlp_kernel<1>, then trust_kernel);
        # its bytes are a prediction's
        sk = kshare["selector"]
        sk["launches_per_prediction"] = 2
        sk["ms_per_prediction"] = 2 * sk["ms_per_launch"]
        sk["algorithmic_bytes_per_prediction"] = sk.pop("algorithmic_bytes_per_launch")
        sk["achieved_gbs"] = sk["algorithmic_bytes_per_prediction"] / (sk["ms_per_prediction"] * 1e-3) / 1e9
    algo = kshare[dom].get("algorithmic_bytes_per_launch", kshare[dom].get("algorithmic_bytes_per_prediction"))
    achieved = kshare[dom]["achieved_gbs"]
    traffic = None
    tf = ROOT / "profiles" / "teno_recon_traffic.json"
    if tf.exists() and dom == "recon":
        t = json.loads(tf.read_text())
        key = "fp32_learned" if learned else prec
        per_cell = t.get("dram_bytes_per_cell_by_form", {}).get(key)
        traffic = per_cell * cells if per_cell else None
    roofline = {"bound": "hbm", "kernel": kernel_names.get(dom, dom), "achieved": achieved, "peak": hbm_peak,
                "unit": "GB/s", "frac": achieved / hbm_peak,
                "peak_source": "MEASURED_PEAKS.json hbm_gbs (measured)" if pk.exists() else "fallback 6800 GB/s",
                "traffic": traffic, "algorithmic_bytes_per_launch": algo,
                "timing": "CUDA events around every launch on the solver's stream (a second pass of W + K steps)"}
    # 11 per step; the selector's inference and neighbour check on the
    # prediction steps (the first of the timed call, then every interval)
    pred_steps = -(-args.steps // max(args.sel_interval, 1)) if learned else 0
    gpu_launches = args.steps * 11 + 2 * pred_steps
    forms[head] = {"value": value, "ms_per_step": ms_max / args.steps, "finite": finite,
                   "kernel_ms_per_launch": {k: v[0] / max(v[1], 1) for k, v in kt.items() if v[1]}}
    if stats:
        forms[head]["selector"] = selector_summary(selector, stats, args.sel_interval)
    if r["tune"]:
        forms[head]["autotune"] = r["tune"]
    solver.close()
    # errors of every form against the plain FP64 path after the same W + K steps
    accuracy = None
    if "fp64" in finals:
        for form, U in finals.items():
            if form != "fp64":
                forms[form].update(errors_vs(m, U, finals["fp64"]))
        if head != "fp64":
            accuracy = {k: forms[head].get(k) for k in ("density_l1_rel_err", "density_linf_rel_err",
                                                        "density_linf_at", "mass_rel_diff", "energy_rel_diff")}
            accuracy["against"] = "plain FP64 GPU path (the reference's operation order), same steps"
            accuracy["bar"] = "density L1 <= 1e-3"
    # the plain FP64 path's binding roof is the FP64 unit: its reconstruction's flops per second
    fp64_roof = None
    fp64_kt = forms.get("fp64", {}).get("kernel_ms_per_launch", {})
    if "recon" in fp64_kt:
        flops_cell = teno_flops_per_cell("fp64")
        fp64_peak = mg.fp64_peak_gflops(local)
        rs = fp64_kt["recon"] * 1e-3
        fp64_roof = {"form": "fp64", "kernel": "teno_kernel<10,20,2>",
                     "achieved_gflops": flops_cell * cells / rs / 1e9, "peak_gflops": fp64_peak,
                     "frac": flops_cell * cells / rs / 1e9 / fp64_peak, "flops_per_cell": flops_cell,
                     "peak_source": "measured FMA-chain probe on this GPU"}

    end_time = run_end_time(args, local, selector) if args.end_time_n >= 0 else None
    c5 = run_c5(args, local, selector) if args.c5_n > 0 else None
    wedge = run_wedge(args, local, selector or load_selector(local)) if args.wedge_n > 0 else None
    batched = run_batched(args, local) if args.batch_cases > 0 else None

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        rate, threads, secs, ccells, csetup, cfin = cpu_oracle_rate(args.cpu_sample_n, 64, 1, args.variant)
        cpu = {"value": rate, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"cartesian_tri {args.cpu_sample_n}x{args.cpu_sample_n} ({ccells} cells) of the same "
                         f"workload, FP64 plain, 64 steps after 1 warm-up, {threads} OpenMP threads, "
                         f"{secs:.1f} s timed (bench.py --impl reference times the full 1024x1024 mesh)",
               "finite": cfin}

    if rank == 0:
        cfg = workload_config(args, args.n)
        line = {"form": head, "precision": prec + (" + learned stencil selector" if learned else ""),
                "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None,
                "dtype": "f32 (reconstruction, flux) + f64 (state, accumulation)" if prec == "fp32" else "f64",
                "data": "synthetic", "config": cfg,
                "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
                "gpu_launches": gpu_launches, "clocks": clk, "roofline": roofline,
                "kernels": kshare, "stage_bytes": stage_bytes, "finite": finite, "status_flags": flags,
                "forms": forms, "setup_s": setup_s, "cpu_baseline": cpu}
        if fp64_roof:
            line["fp64_roof"] = fp64_roof
        if accuracy:
            line["accuracy_vs_fp64"] = accuracy
        for key, sec in (("end_time", end_time), ("c5", c5), ("wedge", wedge), ("batched", batched)):
            if sec:
                line[key] = sec
        print(json.dumps(line), flush=True)
    reps.close()


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
