"""Train the learned TENO stencil selector on the GPU and save its weights.

    python -m mallard_gb300.train_selector [--out PATH] [--quick]

Training pairs are harvested from the FP64 solver's own runs (corrected
TENO, p = 3, HLLC, SSPRK3, CFL 0.5) at seeded random initial states of
four problem families:
  * Sod-type shock tubes on a 1000 x 8 strip of triangles (symmetry
    boundaries), random left/right states and diaphragm position;
  * two-dimensional four-quadrant Riemann problems on the unit square
    (transmissive boundaries), random quadrant states and split point,
    harvested over the first steps;
  * cylindrical explosions (random centre, radius and states);
  * supersonic flow through a ramp channel (Delaunay mesh, random ramp
    angle and Mach number, Rusanov flux), harvested every 100 steps.
Each harvest keeps every cell where some variable leaves the central
stencil and a fraction of the all-central cells.  The network is then
trained with minibatch Adam by the library's own kernels.  --big runs the
large harvest (about 50M rows): the robust TENO variant, 512 x 512
four-quadrant and explosion runs of 600 steps, longer shock tubes, more
ramp channels.
"""

import argparse
import time
from pathlib import Path

import numpy as np

from . import Mesh, Solver, state_from_primitives
from .selector import Selector, default_weights_path

GAS = dict(gamma=1.4, p_ref=101325.0, T_ref=298.15, rho_ref=1.225)


def _solver(mesh, bc, variant="corrected"):
    blist = [{"name": z, "type": bc} for z in mesh.zone_names[1:]]
    return Solver(mesh, face_reconstruction="TENO", basis_type="legendre", basis_order=3, riemann_solver="HLLC",
                  boundaries=blist, teno_variant=variant, precision="fp64_fast", **GAS)


def _run_and_harvest(sel, mesh, bc, U, W, steps, every, keep, seed, variant="corrected"):
    rows = 0
    with _solver(mesh, bc, variant) as s:
        s.set_state(U, W)
        for k in range(steps // every):
            s.run(0.5, every)
            if s.status() != 0:
                break
            rows += sel.harvest(s, keep_central=keep, seed=seed * 1000 + k)
    return rows


def harvest_all(sel, seed=0, quick=False, log=print):
    r = np.random.default_rng(seed)
    rows = 0
    # shock tubes, 1000 x 8 strip (a one-cell strip makes the p = 3 least-squares
    # systems degenerate)
    strip = Mesh.generate("cartesian_tri", 1000, 8, 1.0, 0.008)
    x = strip.cell_coords[:, 0]
    for i in range(4 if quick else 16):
        left = (r.uniform(0.5, 2.0), r.uniform(-0.5, 0.5), r.uniform(0.5, 2.0))
        right = (r.uniform(0.05, 0.5), r.uniform(-0.5, 0.5), r.uniform(0.05, 0.5))
        if r.random() < 0.5:
            left, right = right, left
        xd = r.uniform(0.3, 0.7)
        sel_l = x < xd
        rho = np.where(sel_l, left[0], right[0])
        u = np.where(sel_l, left[1], right[1])
        p = np.where(sel_l, left[2], right[2])
        U, W = state_from_primitives(rho, u, 0 * u, p, **GAS)
        rows += _run_and_harvest(sel, strip, "symmetry", U, W, 200, 40, 0.05, 10 + i)
    log(f"  shock tubes: {rows} rows")
    # four-quadrant problems
    n = 128 if quick else 256
    sq = Mesh.generate("cartesian_tri", n, n, 1.0, 1.0)
    cx, cy = sq.cell_coords[:, 0], sq.cell_coords[:, 1]
    for i in range(2 if quick else 6):
        sx, sy = r.uniform(0.3, 0.8, 2)
        q = [(r.uniform(0.1, 2.0), r.uniform(-1.5, 1.5), r.uniform(-1.5, 1.5), r.uniform(0.03, 2.0)) for _ in range(4)]
        prim = np.zeros((sq.n_cells, 4))
        for k, m in enumerate(((cx >= sx) & (cy >= sy), (cx < sx) & (cy >= sy), (cx < sx) & (cy < sy),
                               (cx >= sx) & (cy < sy))):
            prim[m] = q[k]
        U, W = state_from_primitives(prim[:, 0], prim[:, 1], prim[:, 2], prim[:, 3], **GAS)
        rows += _run_and_harvest(sel, sq, "extrapolation", U, W, 40, 10, 0.05, 100 + i)
    log(f"  + four-quadrant: {rows} rows")
    # cylindrical explosions
    for i in range(2 if quick else 6):
        c = r.uniform(0.3, 0.7, 2)
        rad = r.uniform(0.1, 0.3)
        inn = (cx - c[0]) ** 2 + (cy - c[1]) ** 2 < rad * rad
        a = (r.uniform(0.5, 2.0), r.uniform(0.5, 2.0))
        b = (r.uniform(0.1, 0.5), r.uniform(0.05, 0.4))
        if r.random() < 0.3:
            a, b = b, a
        rho = np.where(inn, a[0], b[0])
        p = np.where(inn, a[1], b[1])
        U, W = state_from_primitives(rho, 0 * rho, 0 * rho, p, **GAS)
        rows += _run_and_harvest(sel, sq, "extrapolation", U, W, 120 if quick else 240, 30, 0.05, 200 + i)
    log(f"  + explosions: {rows} rows")
    # supersonic ramp channels (Rusanov flux, inflow / outflow / slip walls)
    for i in range(1 if quick else 4):
        rows += _run_wedge(sel, r, quick, 300 + i)
    log(f"  + wedges: {rows} rows")
    return rows


def wedge_viscosity(mach=2.5, rho=1.4, p=1.0, reynolds=1e5, length=1.0, prandtl=0.72):
    """Viscous parameters of the ramp channel: mu at the inflow temperature
    from the Reynolds number on the ramp length, Sutherland's law with the
    air ratio S / T_inf = 110.4 / 288.15."""
    R = GAS["p_ref"] / (GAS["T_ref"] * GAS["rho_ref"])
    u = mach * float(np.sqrt(GAS["gamma"] * p / rho))
    T = p / (rho * R)
    return {"mu_ref": rho * u * length / reynolds, "T_mu_ref": T, "sutherland_S": T * 110.4 / 288.15,
            "prandtl": prandtl}


def wedge_setup(mesh, mach=2.5, rho=1.4, p=1.0, riemann="Rusanov", precision="fp64_fast", reynolds=None,
                teno_variant="corrected", gradients="recon"):
    """Solver and initial state of the supersonic ramp channel: uniform inflow
    state everywhere, "upt" inflow, "p_out" outflow, walls (slip; no-slip
    and viscous when a Reynolds number is given, with the viscous flux's
    cell gradients from `gradients`: "recon" or "green_gauss")."""
    R = GAS["p_ref"] / (GAS["T_ref"] * GAS["rho_ref"])
    u = mach * float(np.sqrt(GAS["gamma"] * p / rho))
    T = p / (rho * R)
    blist = [{"name": "inflow", "type": "upt", "u": [u, 0.0], "p": p, "T": T},
             {"name": "outflow", "type": "p_out", "p": p},
             {"name": "wall", "type": "wall_adiabatic"}, {"name": "top", "type": "wall_adiabatic"}]
    visc = dict(wedge_viscosity(mach, rho, p, reynolds), gradients=gradients) if reynolds else None
    s = Solver(mesh, face_reconstruction="TENO", basis_type="legendre", basis_order=3, riemann_solver=riemann,
               boundaries=blist, teno_variant=teno_variant, precision=precision, viscous=visc, **GAS)
    n = mesh.n_cells
    U, W = state_from_primitives(np.full(n, rho), np.full(n, u), np.zeros(n), np.full(n, p), **GAS)
    return s, U, W


def _run_wedge(sel, r, quick, seed):
    mesh = Mesh.ramp_channel(150 if quick else 240, 50 if quick else 80, 3.0, 1.0, 0.5, r.uniform(8.0, 20.0), 0.2,
                             seed=seed)
    s, U, W = wedge_setup(mesh, mach=r.uniform(1.8, 3.5))
    rows = 0
    with s:
        s.set_state(U, W)
        for k in range(4):
            s.run(0.4, 50 if quick else 100)
            if s.status() != 0:
                break
            rows += sel.harvest(s, keep_central=0.05, seed=seed * 1000 + k)
    return rows


def harvest_big(sel, seed=0, log=print):
    """The large harvest (about 50M rows): the same four families with the
    robust TENO variant, which keeps the four-quadrant problems finite to
    their later, more varied states, on larger meshes and longer runs."""
    r = np.random.default_rng(seed)
    rows = 0
    strip = Mesh.generate("cartesian_tri", 1000, 8, 1.0, 0.008)
    x = strip.cell_coords[:, 0]
    for i in range(48):
        left = (r.uniform(0.5, 2.0), r.uniform(-0.5, 0.5), r.uniform(0.5, 2.0))
        right = (r.uniform(0.05, 0.5), r.uniform(-0.5, 0.5), r.uniform(0.05, 0.5))
        if r.random() < 0.5:
            left, right = right, left
        sel_l = x < r.uniform(0.3, 0.7)
        rho = np.where(sel_l, left[0], right[0])
        u = np.where(sel_l, left[1], right[1])
        p = np.where(sel_l, left[2], right[2])
        U, W = state_from_primitives(rho, u, 0 * u, p, **GAS)
        rows += _run_and_harvest(sel, strip, "symmetry", U, W, 800, 40, 0.05, 10 + i, "robust")
    log(f"  shock tubes: {rows} rows")
    sq = Mesh.generate("cartesian_tri", 512, 512, 1.0, 1.0)
    sq.permute_cells(seed + 1)
    cx, cy = sq.cell_coords[:, 0], sq.cell_coords[:, 1]
    for i in range(24):
        sx, sy = r.uniform(0.3, 0.8, 2)
        q = [(r.uniform(0.1, 2.0), r.uniform(-1.5, 1.5), r.uniform(-1.5, 1.5), r.uniform(0.03, 2.0)) for _ in range(4)]
        prim = np.zeros((sq.n_cells, 4))
        for k, m in enumerate(((cx >= sx) & (cy >= sy), (cx < sx) & (cy >= sy), (cx < sx) & (cy < sy),
                               (cx >= sx) & (cy < sy))):
            prim[m] = q[k]
        U, W = state_from_primitives(prim[:, 0], prim[:, 1], prim[:, 2], prim[:, 3], **GAS)
        rows += _run_and_harvest(sel, sq, "extrapolation", U, W, 600, 20, 0.05, 100 + i, "robust")
        log(f"  four-quadrant {i + 1}/24: {rows} rows")
    for i in range(8):
        c = r.uniform(0.3, 0.7, 2)
        rad = r.uniform(0.1, 0.3)
        inn = (cx - c[0]) ** 2 + (cy - c[1]) ** 2 < rad * rad
        a = (r.uniform(0.5, 2.0), r.uniform(0.5, 2.0))
        b = (r.uniform(0.1, 0.5), r.uniform(0.05, 0.4))
        if r.random() < 0.3:
            a, b = b, a
        rho = np.where(inn, a[0], b[0])
        p = np.where(inn, a[1], b[1])
        U, W = state_from_primitives(rho, 0 * rho, 0 * rho, p, **GAS)
        rows += _run_and_harvest(sel, sq, "extrapolation", U, W, 600, 30, 0.05, 200 + i, "robust")
    log(f"  + explosions: {rows} rows")
    for i in range(8):
        rows += _run_wedge(sel, r, False, 300 + i)
    log(f"  + wedges: {rows} rows")
    return rows


def train(out=None, seed=0, quick=False, epochs=None, log=print, big=False):
    t0 = time.time()
    sel = Selector(seed=seed + 1)
    rows = harvest_big(sel, seed=seed, log=log) if big else harvest_all(sel, seed=seed, quick=quick, log=log)
    t1 = time.time()
    epochs = epochs or (6 if quick else 12)
    losses = sel.train(epochs=epochs, batch=4096, lr=2e-3, seed=seed + 2)
    t2 = time.time()
    log(f"harvest {rows} rows in {t1 - t0:.1f} s; train {epochs} epochs in {t2 - t1:.1f} s; "
        f"loss {losses[0]:.4f} -> {losses[-1]:.4f}")
    if out:
        Path(out).parent.mkdir(parents=True, exist_ok=True)
        sel.save(out, rows=rows, losses=losses, seed=seed, epochs=epochs)
    return sel, losses


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=str(default_weights_path()))
    ap.add_argument("--seed", type=int, default=20261203)
    ap.add_argument("--quick", action="store_true")
    ap.add_argument("--epochs", type=int, default=None)
    ap.add_argument("--big", action="store_true", help="the large harvest (about 50M rows, robust TENO runs)")
    a = ap.parse_args()
    train(a.out, seed=a.seed, quick=a.quick, epochs=a.epochs, big=a.big)


if __name__ == "__main__":
    main()
