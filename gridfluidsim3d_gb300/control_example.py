"""Differentiable control at scale: Adam on the per-particle initial velocities of
the 128^3 dam-break particle layout (8 particles per cell, fluid box at rest
against the walls, no gravity by default) so that the centroid of the fluid
follows a target trajectory over 60 substeps of 1/30 s.

With gravity (--gravity -25) the dam break is dominated by discrete events --
floor and wall collisions of the particles every substep, compaction and the
per-cell cap -- and its loss is not a differentiable function of the initial
velocities (central differences change sign with the step size), so the
default problem is the smooth one.

    python -m gridfluidsim3d_gb300.control_example --iterations 50

Each iteration runs the forward rollout (every substep's particle state and
pressure checkpointed on the device) and the hand-written CUDA adjoint
(gridfluidsim3d_gb300.autograd), then one Adam step.  The target trajectory is
the uncontrolled centroid path shifted by `--shift` cells in +x growing
linearly over the rollout.  Prints one JSON line per iteration (loss, forward
and backward device ms) and a summary line with the peak device memory.
"""
from __future__ import annotations

import argparse
import json
import time

import torch

from . import PRECISION_MIXED, FluidSimulation, scenes
from .autograd import FlipRollout


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--grid", type=int, default=128)
    ap.add_argument("--iterations", type=int, default=50)
    ap.add_argument("--lr", type=float, default=0.05)
    ap.add_argument("--shift", type=float, default=4.0, help="cells in +x at the end of the rollout")
    ap.add_argument("--gravity", type=float, default=0.0, help="y body force (m/s^2)")
    a = ap.parse_args(argv)
    dev = torch.device("cuda", 0)
    db = scenes.dam_break(a.grid)
    steps = int(db.meta["substeps"])
    sim = FluidSimulation(*db.dims, db.dx, max_particles=db.num_particles)
    sim.precision = PRECISION_MIXED
    sim.reset_body_force()
    sim.add_body_force(0.0, a.gravity, 0.0)
    sim.set_material_grid(db.mat)
    roll = FlipRollout(sim, steps, db.dt, db.num_particles)
    x0 = torch.tensor(db.pos, device=dev)
    v = torch.zeros((db.num_particles, 3), device=dev, requires_grad=True)
    with torch.no_grad():
        _, base = roll(x0, velocities=v)   # the uncontrolled centroid path
    ramp = torch.linspace(0.0, 1.0, steps + 1, device=dev)[:, None]
    goal = base + ramp * torch.tensor([a.shift * db.dx, 0.0, 0.0], device=dev)
    opt = torch.optim.Adam([v], lr=a.lr)
    free_low = torch.cuda.mem_get_info(dev)[0]
    t0 = time.time()
    first = None
    for it in range(a.iterations):
        opt.zero_grad()
        _, cen = roll(x0, velocities=v)
        loss = ((cen - goal) ** 2).sum()
        loss.backward()
        opt.step()
        fwd_ms, bwd_ms, _ = roll.info()
        free_low = min(free_low, torch.cuda.mem_get_info(dev)[0])
        val = float(loss.detach())
        first = val if first is None else first
        print(json.dumps({"iteration": it, "loss": val, "forward_ms": round(fwd_ms, 1),
                          "backward_ms": round(bwd_ms, 1),
                          "centroid_end_x_cells": float(cen[-1, 0].detach() / db.dx)}), flush=True)
    total = torch.cuda.mem_get_info(dev)[1]
    print(json.dumps({"summary": True, "particles": db.num_particles, "substeps": steps,
                      "iterations": a.iterations, "loss_first": first, "loss_last": val,
                      "wall_s": round(time.time() - t0, 1), "peak_device_bytes": int(total - free_low)}), flush=True)
    roll.close()
    sim.close()


if __name__ == "__main__":
    main()
