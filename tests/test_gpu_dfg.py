"""The DFG (Schäfer-Turek) 2D cylinder benchmark at Re = 20 as the reference runs it
(benchmarks/Cylinder2D/CylinderFlow_Re20.mojo): a 5N x N channel of height L = 0.41 (dx = L/(N-1)),
parabolic moving-wall inlet of mean velocity 0.2 (0.01 in lattice units), equilibrium outlet,
no-slip walls, a cylinder of radius 0.05 centred on the node nearest (0.2, 0.2), DDF shift, drag by
momentum exchange over the cylinder's boundary nodes.  The drag coefficient after the reference's
800,000 steps (400,000 at N = 256) must match the DFG value within the discretisation error the
reference records for the same resolution, and the reference's own recorded drag within 0.5 %.
Targets come from tests/golden/dfg_re20.json (make_dfg_fixture.py extracts them from the
reference's benchmark file)."""
from __future__ import annotations

import json
import math
from pathlib import Path

import numpy as np
import pytest
import torch

from mojo_lbm_gb300 import Flags, LBM_Config, LBM_Grid, LBM_method, get_D2Q9, preprocess
from mojo_lbm_gb300.geometry import get_sphere_boundary_indices
from mojo_lbm_gb300.solver import Solver

pytestmark = pytest.mark.gpu

FIXTURE = json.loads((Path(__file__).parent / "golden" / "dfg_re20.json").read_text())


def dfg_drag(N: int, coll: str, steps: int, chunk: int = 100_000):
    """(Cd, Cl) of the reference's DFG Re = 20 set-up at resolution N after `steps` steps, and the
    Cd of each chunk."""
    L, U_phys, U_lat, radius = 0.41, 0.2, 0.01, 0.05
    dx = L / (N - 1)
    grid = LBM_Grid(get_D2Q9(), 5 * N, N, 1, (16, 16, 1), dx=dx)
    cfg = LBM_Config(LBM_method.DOUBLE_BUFFER, BCs={Flags.EQUILIBRIUM}, DDF_shift=True, collision_op=coll)
    units = grid.get_UnitSystem_with_Re(U_phys, U_lat, 2 * radius, 20.0)
    n = grid.num_points
    flags, bc = np.zeros(n, np.uint8), np.zeros(n * 3, np.float32)
    Um = 1.5 * U_phys
    preprocess.set_exterior_walls(grid, cfg, flags, bc, "+X", Flags.EQUILIBRIUM, [], 1.0)
    preprocess.set_exterior_walls_with_func(grid, cfg, flags, bc, "-X", Flags.SOLID,
                                            lambda x, y, z: [4 * Um * y * (L - y) / (L * L), 0.0 * y],
                                            unitSystem=units, rho=1.0)
    preprocess.set_exterior_walls(grid, cfg, flags, bc, "-Y", Flags.SOLID, [0.0, 0.0], 1.0)
    preprocess.set_exterior_walls(grid, cfg, flags, bc, "+Y", Flags.SOLID, [0.0, 0.0], 1.0)
    c = math.floor(0.2 / dx) * dx  # the reference's 0.2 // dx: the centre on a node
    ids = get_sphere_boundary_indices(grid, flags, [c, c, 0.0], radius)
    solver = Solver(grid, cfg)
    fa = torch.zeros(n * 9, device="cuda")  # DDF-shifted rest state
    fb = torch.zeros_like(fa)
    bct, flt = torch.from_numpy(bc).cuda(), torch.from_numpy(flags).cuda()
    idt = torch.from_numpy(ids.astype(np.int32)).cuda()
    force = torch.zeros(len(ids) * 2, device="cuda")
    scale = 2 * units.force.C_lat_to_phys() / (U_phys ** 2 * 2 * radius)
    history, done = [], 0
    while done < steps:
        solver.run(fa, fb, bct, flt, units.tau, chunk, done)
        done += chunk
        solver.drag_force(force, fa, flt, idt)  # after an even number of steps fa is current
        fn = force.double().cpu().numpy()
        history.append(float(fn[:len(ids)].sum() * scale))
    solver.close()
    return history[-1], float(fn[len(ids):].sum() * scale), history


def _recorded(grid, coll):
    for r in FIXTURE["reference_runs"]:
        if r["grid"] == grid and r["collision"] in (coll, "not stated"):
            return r
    raise KeyError(grid)


@pytest.mark.parametrize("N,coll,steps,grid,tol_dfg", [(256, "SRT", 400_000, [1024, 256], 0.015),
                                                        (256, "KBC", 400_000, [1024, 256], 0.015),
                                                        (512, "SRT", 800_000, [2560, 512], 0.003)])
def test_dfg_cylinder_re20_drag(N, coll, steps, grid, tol_dfg):
    cd, cl, history = dfg_drag(N, coll, steps)
    ref = _recorded(grid, coll)
    print(f"\nN={N} {coll}: Cd {cd:.5f} (DFG {FIXTURE['Cd']:.5f}, reference run {ref['drag']:.5f}), "
          f"Cl {cl:.5f}; Cd per 100k steps {['%.4f' % v for v in history]}")
    assert abs(history[-1] - history[-2]) < 2e-3 * cd, "drag not converged"
    assert abs(cd - FIXTURE["Cd"]) / FIXTURE["Cd"] < tol_dfg
    assert abs(cd - ref["drag"]) / ref["drag"] < 5e-3
    assert 0.0 < cl < 0.03  # the lift is small and positive (DFG 0.0106; the reference 0.012-0.013)
