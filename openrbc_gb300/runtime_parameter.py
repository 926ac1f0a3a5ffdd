"""Host-side mirror of OpenRBC's run-time parameters (src/runtime_parameter.h:38-144).

Same option names (short and long), same defaults and the same validation as
RTParameter, plus the options of the GPU step (precision, integrator, skin,
batch file, autotune).  The reference's compile-time switches LANGEVIN /
FUSED_INTEGRATOR and `real` (src/config_static.h:30-34) become --integrator and
--precision.  Values convert like C's atoi / atof (leading numeric prefix,
0 when there is none).  The reference registers "-r" twice (rho at :102 and
random-seed at :107), so "-r X" sets both; --rho and --random-seed are the
unambiguous spellings.  This is kept so command lines behave identically.
"""
from __future__ import annotations

import re
import sys
from dataclasses import dataclass, field
from typing import List, Optional


def _atoi(s: str) -> int:
    m = re.match(r"\s*[+-]?\d+", s)
    return int(m.group(0)) if m else 0


def _atof(s: str) -> float:
    m = re.match(r"\s*[+-]?(\d+\.?\d*([eE][+-]?\d+)?|\.\d+([eE][+-]?\d+)?|inf|nan)", s, re.I)
    return float(m.group(0)) if m else 0.0


class ParameterError(ValueError):
    """Raised where the reference calls rt_assert (src/util_misc.h:54-59), which prints and exits."""


# (attribute, short, long, converter, help) in the reference's registration order (:84-107)
_OPTIONS = [
    ("init", "i", "init", str, "Model initialization mode, must be 'lipid' or 'vesicle' or 'trimesh'"),
    ("mesh", "m", "mesh", str, "Prefix for the 3 mesh files"),
    ("t_total", "t", "total-time", _atof, "Total time in simulation units"),
    ("dt", "k", "dt", _atof, "Simulation time step size"),
    ("eta", "e", "eta", _atof, "Solvent viscosity for Langevin integrator"),
    ("stray_tolerance", "", "stray-tolerance", _atof, "Stray lipid tolerance (multiples of the median)"),
    ("opt_nstep", "E", "opt-nstep", _atoi, "Number of optimization steps"),
    ("dr_opt", "", "opt-max-move", _atof, "Maximum displacement per optimization step"),
    ("dn_opt", "", "opt-max-rotate", _atof, "Maximum rotation per optimization step"),
    ("freq_voronoi", "V", "voronoi-update-freq", _atoi, "Frequency (#steps) of Voronoi cell update"),
    ("freq_sort_ctrd", "", "centroid-reorder-freq", _atoi, "Frequency (#steps) of centroid reorder"),
    ("freq_sort_bond", "", "bond-reorder-freq", _atoi, "Frequency (#steps) of bond locality maintenance"),
    ("freq_display", "D", "display-frequency", _atoi, "Frequency (#steps) of screen info display"),
    ("freq_dump", "d", "dump-frequency", _atoi, "Frequency (#steps) of trajectory file output"),
    ("freq_sort_bond", "", "bond-sort-frequency", _atoi, "Frequency (#steps) to reorder bonds"),
    ("freq_cleanup", "", "cleanup-frequency", _atoi, "Frequency (#steps) to remove stray lipid particles"),
    ("dump_field", "", "dump-field", _atoi, "Fields to dump: 1 position, 2 rotation, 4 voronoi, 8 velocity, 16 force"),
    ("Q", "Q", "nose-hoover-Q", _atof, "Nose-Hoover relaxation parameter"),
    ("rho", "r", "rho", _atof, "Lipid number density"),
    ("kBT", "T", "kBT", _atof, "Thermal noise level"),
    ("voronoi_cell_size", "", "voronoi-cell-size", _atoi, "Average size (#lipids) of Voronoi cells"),
    ("file_topo", "o", "topology-file", str, "Filename for saving topology"),
    ("file_traj", "x", "trajectory-file", str, "Filename for saving trajectory"),
    ("rseed", "r", "random-seed", _atoi, "Seed for random number generation"),
    # GPU step options (no reference counterpart)
    ("gpu", "", "gpu", _atoi, "Run the time step on the GPU (1) or report the host path (0)"),
    ("precision", "", "precision", str, "GPU arithmetic: 'mixed' (FP32 forces, FP64 reductions) or 'fp64'"),
    ("integrator", "", "integrator", str, "'langevin' (default build) or 'nose-hoover' (LANGEVIN undefined)"),
    ("skin", "", "skin", _atof, "Neighbour-list skin; rebuild when a particle moved more than skin/2"),
    ("rebuild_every", "", "rebuild-every", _atoi, "Also rebuild the neighbour list every k steps (0 = off)"),
    ("batch_file", "", "batch-file", str, "Batch description (systems to advance in one launch)"),
    ("autotune", "", "autotune", _atoi, "Pick skin / rebuild cadence by timing short trials (1 = on)"),
]


@dataclass
class RTParameter:
    init: str = "vesicle"
    mesh: str = ""
    voronoi_cell_size: int = 14
    rho: float = 1.05
    kBT: float = 0.22
    eta: float = 0.01
    stray_tolerance: float = 2.5
    t_total: float = 10.0
    dt: float = 1e-2
    opt_nstep: int = 1000
    dr_opt: float = 5e-2
    dn_opt: float = 5e-2
    freq_voronoi: int = 2
    freq_sort_ctrd: int = 24
    freq_sort_bond: int = 120
    freq_cleanup: int = 60
    nstep: int = 0
    rseed: int = 0xBAD5EED
    freq_display: int = 100
    freq_dump: int = 10000
    dump_field: int = 1 + 2 + 4
    file_topo: str = "cell.data"
    file_traj: str = "cell.orbc"
    Q: float = 0.0
    zeta: float = 0.0
    box: List[List[float]] = field(default_factory=lambda: [[-1000.0, 1000.0] for _ in range(3)])
    # GPU step
    gpu: int = 1
    precision: str = "mixed"
    integrator: str = "langevin"
    skin: float = 0.4
    rebuild_every: int = 0
    batch_file: str = ""
    autotune: int = 0

    @property
    def bsize(self):
        return [b[1] - b[0] for b in self.box]

    def set_Q(self, n: int) -> None:  # src/runtime_parameter.h:76
        self.Q = n * 0.01

    @classmethod
    def from_argv(cls, argv: Optional[List[str]] = None, quiet: bool = True) -> "RTParameter":
        """Parse like RTParameter::parse (src/runtime_parameter.h:123-143): each
        option is looked up in argv in registration order; every occurrence of
        its short or long form followed by a value sets it (the last one wins)."""
        argv = list(sys.argv[1:] if argv is None else argv)
        p = cls()
        for attr, short, long, cvt, _help in _OPTIONS:
            for i, tok in enumerate(argv[:-1]):
                if (short and tok == "-" + short) or tok == "--" + long:
                    setattr(p, attr, cvt(argv[i + 1]))
                    if not quiet:
                        print(f"From command line: {long:25s} = {argv[i + 1]}")
        p.validate()
        return p

    def validate(self) -> None:  # src/runtime_parameter.h:116-120
        if self.init not in ("lipid", "vesicle", "trimesh"):
            raise ParameterError("Initialization mode must be 'lipid', 'vesicle', or 'trimesh'")
        if self.init == "trimesh" and not self.mesh:
            raise ParameterError("Initialization mode 'trimesh' specified, but mesh files are not given")
        if self.freq_sort_ctrd % self.freq_voronoi:
            raise ParameterError("Voronoi centroid reorder frequency must be a multiple of voronoi update frequency")
        if self.freq_sort_bond % self.freq_voronoi:
            raise ParameterError("bond reorder frequency must be a multiple of voronoi update frequency")
        if self.freq_cleanup % self.freq_voronoi:
            raise ParameterError("stray lipid cleanup frequency must be a multiple of voronoi update frequency")
        if self.precision not in ("mixed", "fp64"):
            raise ParameterError("precision must be 'mixed' or 'fp64'")
        if self.integrator not in ("langevin", "nose-hoover"):
            raise ParameterError("integrator must be 'langevin' or 'nose-hoover'")
        if not self.dt > 0:
            raise ParameterError("dt must be positive")
        if self.skin < 0:
            raise ParameterError("skin must be non-negative")

    @staticmethod
    def help() -> str:
        lines = []
        for _attr, short, long, _cvt, text in _OPTIONS:
            lines.append(f"{('-' + short) if short else '':6s}{'--' + long:25s}   {text}")
        return "\n".join(lines)
