"""GB300-native engine for the gpvmc Metropolis sampling path.

The compute path is the C-ABI library built from gpvmc_gb300/csrc (CUDA for
sm_103a, C++ host); this package is its Python host side.  See
gpvmc_gb300.vmc for the reference-named API.
"""
from ._lib import GvError, lib  # noqa: F401
from .vmc import (Job, LatticeStepper, MetroMC, ProjHeis, SlaterDeterminant, SquareLattice,  # noqa: F401
                  StagFluxGroundState, StagFluxTransExciton, StagFluxLongExciton, StagMagnTrack, StagMagnZ, StatSpinStruct, OverlapTrack, pi_phi)
from .serving import Server  # noqa: F401
from .output import FileManager, convert_tree, save_quantities, write_wavefunction  # noqa: F401

__version__ = "0.1.0"
