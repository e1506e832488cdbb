"""Input containers mirroring the reference's data for the tracking path.

``Grid``    -- structured MODFLOW 6 DIS grid (RectangularGridDisMf6.f90:122-360)
``Flow``    -- one flow/transport time step: FLOW-JA-FACE in IA/JA form plus
               the per-cell arrays of FlowModelData / TransportModelData
``Options`` -- RWOPTS / DSP / simulation options (ParticleTrackingOptions.f90)
``Particles`` -- the particle arrays of a particle group (Particle.f90:7-17)

All arrays are numpy, in the reference's conventions: 1-based cell numbers,
1-based IA/JA, FLOW-JA-FACE positive into the cell.
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import Optional

import numpy as np

# time step kinds (ModpathSimulationData.f90, RWOPTS)
ADV, DISP, MIN_ADV_DISP, FIXED = 1, 2, 3, 4
# advection kinds
EXPONENTIAL, EULERIAN = 1, 2
# precision of the GPU path
FP64, MIXED = 0, 1
# driver status codes (MPathRW.F90:1337-1403)
PENDING, ACTIVE, BOUNDARY, WEAK_SINK, WEAK_SOURCE, NO_EXIT, STOP_ZONE, INACTIVE, UNRELEASED, UNDEFINED = range(10)


@dataclass
class Grid:
    nlay: int
    nrow: int
    ncol: int
    delr: np.ndarray  # (ncol,)
    delc: np.ndarray  # (nrow,)
    top: np.ndarray   # (nrow*ncol,)
    botm: np.ndarray  # (nlay*nrow*ncol,)

    @property
    def ncell(self) -> int:
        return self.nlay * self.nrow * self.ncol

    def node(self, k, i, j):
        """1-based node number of 0-based (layer, row, column)."""
        return k * self.nrow * self.ncol + i * self.ncol + j + 1


@dataclass
class Flow:
    ia: np.ndarray
    ja: np.ndarray
    flowja: np.ndarray
    porosity: np.ndarray
    retardation: np.ndarray
    iboundts: np.ndarray
    alpha_l: np.ndarray
    alpha_t: np.ndarray
    dm_eff: np.ndarray
    uniform_dispersion: bool = True
    steady_state: bool = True
    default_icbound: int = 1
    icboundts: Optional[np.ndarray] = None
    boundary_flows: Optional[np.ndarray] = None
    heads: Optional[np.ndarray] = None
    celltype: Optional[np.ndarray] = None
    source_flow: Optional[np.ndarray] = None
    sink_flow: Optional[np.ndarray] = None
    zones: Optional[np.ndarray] = None
    alpha_lv: Optional[np.ndarray] = None   # axisymmetric model: vertical dispersivities
    alpha_tv: Optional[np.ndarray] = None   # (None: equal to alpha_l / alpha_t)


@dataclass
class Options:
    time_step_kind: int = ADV
    ts_param: tuple = (0.1, 0.1)
    advection_kind: int = EULERIAN
    dim_mask: tuple = (1, 1, 1)
    dispersion_model: int = 0
    stop_weak_sinks: bool = False
    stop_weak_sources: bool = False
    backward: bool = False
    stop_zone: int = 0
    uniform_porosity: bool = True
    rng_seed: int = 0x5EED
    precision: int = FP64


@dataclass
class Particles:
    cell: np.ndarray            # int32, 1-based
    lx: np.ndarray
    ly: np.ndarray
    lz: np.ndarray
    t: np.ndarray
    status: np.ndarray          # int32
    mass: Optional[np.ndarray] = None
    id: Optional[np.ndarray] = None        # uint64 Philox key per particle
    rng_ctr: Optional[np.ndarray] = None   # uint64 Philox block counter

    @property
    def n(self) -> int:
        return int(self.cell.shape[0])

    def copy(self) -> "Particles":
        def c(a):
            return None if a is None else np.array(a, copy=True)
        return Particles(c(self.cell), c(self.lx), c(self.ly), c(self.lz), c(self.t), c(self.status),
                         c(self.mass), c(self.id), c(self.rng_ctr))
