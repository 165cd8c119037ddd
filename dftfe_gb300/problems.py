"""Seeded synthetic Kohn-Sham problems for the CheFSI path.

DFT-FE publishes no CheFSI benchmark inputs; these generators stand in with the shapes,
sizes and value distributions of the workloads the path is measured on:

* ``workload_small``  -- periodic cube L=15 bohr, 10^3 cells, degree 4 (64,000 dofs),
  8 Gaussian wells (centres U[0,L)^3, depth U(1,3) Ha, width 1 bohr), 96 wavefunctions
  (48 occupied), Chebyshev degree 24, FP64;
* ``workload_mixed``  -- L=30, 20^3 cells, degree 6 (1,728,000 dofs), 64 wells with 8
  Gaussian projectors each (radius 3 bohr, couplings U(-0.5, 0.5) Ha), 1024 wavefunctions,
  Chebyshev degree 30;
* ``workload_adjoint`` -- the small operator with 256 wavefunctions (lowest 128 summed);
* ``workload_bloch``  -- complex Bloch Hamiltonians (k uniform in the first Brillouin zone)
  on 6^3..14^3 meshes at degree 4, 64..512 wavefunctions, 4..16 wells;
* ``workload_large``  -- L=48, 32^3 cells, degree 5 (4,096,000 dofs), 256 wells x 8
  projectors, 4096 wavefunctions in blocks of 256, degree 40.

Random streams: ``numpy.random.default_rng(seed)`` for the potential/projectors and
``default_rng(seed + 1)`` for X0 ~ U(-1, 1).
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from . import fe


@dataclass
class Problem:
    name: str
    mesh: fe.PeriodicCubeMesh
    cell_map: np.ndarray            # [n_cells, n_e] int32
    cell_mats: np.ndarray           # [n_cells, n_e, n_e] float64 or complex128 (applied form)
    mass: np.ndarray                # lumped mass [n_dofs]
    nonlocal_: fe.NonlocalProjectors | None
    n_wfc: int
    cheb_degree: int
    n_occupied: int
    kpoint: np.ndarray | None = None
    seed: int = 0
    info: dict = field(default_factory=dict)

    @property
    def n_dofs(self) -> int:
        return self.mesh.n_dofs

    @property
    def sqrt_mass(self) -> np.ndarray:
        return np.sqrt(self.mass)

    @property
    def inv_sqrt_mass(self) -> np.ndarray:
        return 1.0 / np.sqrt(self.mass)

    @property
    def is_complex(self) -> bool:
        return np.iscomplexobj(self.cell_mats)

    def initial_vectors(self, n_wfc: int | None = None) -> np.ndarray:
        n = self.n_wfc if n_wfc is None else n_wfc
        rng = np.random.default_rng(self.seed + 1)
        X = rng.uniform(-1.0, 1.0, (self.n_dofs, n))
        if self.is_complex:
            X = X + 1j * rng.uniform(-1.0, 1.0, (self.n_dofs, n))
        return X


def make_problem(n: int, L: float, p: int, n_wells: int, n_wfc: int, seed: int = 0,
                 cheb_degree: int = 24, n_occupied: int | None = None, projectors: bool = False,
                 kpoint=None, depth=(1.0, 3.0), width: float = 1.0, proj_rcut: float = 3.0,
                 name: str = "custom", with_cell_mats: bool = True) -> Problem:
    mesh = fe.PeriodicCubeMesh(n, L, p)
    rng = np.random.default_rng(seed)
    centres = rng.uniform(0.0, L, (n_wells, 3))
    depths = rng.uniform(depth[0], depth[1], n_wells)
    couplings = rng.uniform(-0.5, 0.5, (n_wells, 8))
    pts, w3 = mesh.quadrature()
    v = fe.gaussian_wells_potential(pts, centres, depths, width, L)
    vjxw = v * w3[None, :]
    cell_mats = fe.cell_hamiltonians(mesh, vjxw, kpoint=kpoint) if with_cell_mats else None
    nl = fe.gaussian_projectors(mesh, centres, couplings, sigma=width, rcut=proj_rcut) if projectors else None
    return Problem(name=name, mesh=mesh, cell_map=mesh.cell_dof_map(), cell_mats=cell_mats,
                   mass=mesh.lumped_mass(), nonlocal_=nl, n_wfc=n_wfc, cheb_degree=cheb_degree,
                   n_occupied=n_wfc // 2 if n_occupied is None else n_occupied,
                   kpoint=None if kpoint is None else np.asarray(kpoint, np.float64), seed=seed,
                   info=dict(centres=centres, depths=depths, vjxw=vjxw, n_wells=n_wells))


WORKLOADS = {
    "small": dict(n=10, L=15.0, p=4, n_wells=8, n_wfc=96, cheb_degree=24, n_occupied=48),
    "mixed": dict(n=20, L=30.0, p=6, n_wells=64, n_wfc=1024, cheb_degree=30, projectors=True),
    "adjoint": dict(n=10, L=15.0, p=4, n_wells=8, n_wfc=256, cheb_degree=24, n_occupied=128),
    "large": dict(n=32, L=48.0, p=5, n_wells=256, n_wfc=4096, cheb_degree=40, projectors=True),
    # the mixed workload's cell type (degree 6, 1.5 bohr cells) on an 8^3 mesh: the size used
    # for detailed kernel profiles (inputs still larger than L2, a few GB on the device)
    "mixed_small": dict(n=8, L=12.0, p=6, n_wells=8, n_wfc=1024, cheb_degree=30, projectors=True),
}


def workload(name: str, seed: int = 0, **over) -> Problem:
    kw = dict(WORKLOADS[name])
    kw.update(over)
    return make_problem(name=name, seed=seed, **kw)


def bloch_set(n_ham: int = 32, seed: int = 0, L_cell: float = 1.5, p: int = 4,
              small: bool = False) -> list[Problem]:
    """Independent complex Bloch Hamiltonians: meshes 6^3..14^3 (even sides) at degree p,
    64..512 wavefunctions, 4..16 wells, k ~ U[-pi/L, pi/L)^3 per Hamiltonian."""
    rng = np.random.default_rng(seed)
    out = []
    for h in range(n_ham):
        n = int(rng.choice([2, 3]) if small else rng.choice([6, 8, 10, 12, 14]))
        L = n * L_cell * (2.0 if small else 1.0)
        nw = int(rng.integers(4, 17))
        nwfc = int(rng.choice([8, 16]) if small else rng.choice([64, 128, 256, 512]))
        k = rng.uniform(-np.pi / L, np.pi / L, 3)
        out.append(make_problem(n=n, L=L, p=p, n_wells=nw, n_wfc=nwfc, seed=seed * 1000 + h,
                                kpoint=k, name=f"bloch{h}"))
    return out
