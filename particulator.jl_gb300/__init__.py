"""particulator_gb300 — GB300 (sm_103a) null-collision Monte Carlo step of
Particulator.jl behind a C ABI, with a Python mirror of the package's
population / collision-table / pusher / run API.

The compute path is the in-tree shared library built by ``build.py``; there
is no CPU fallback.
"""
from . import _lib, constants, data
from ._lib import (ELECTRON, PHOTON, POSITRON, PCLError, lib, LIB_PATH)
from .processes import (Moller, RBEB, SeltzerBerger, RelativisticCoulomb, Compton, KleinNishinaCompton,
                        PhotoElectric, BetheHeitler, Bhaba, Bhabha, PositronAnihilation, PositronAnnihilation,
                        N2_ORBITALS, O2_ORBITALS, ORBITALS, totalcs, Elastic, Excitation, NullCollision, Ionization,
                        Attachment)
from .tables import (Electron, Photon, Positron, BinaryIntervals, ChebyshevCollisionTable,
                     collision_table_from_processes, ContinuumLoss, ChebContinuumLoss, speed,
                     momentum_norm_from_kin, precheb, CollisionTable, lxcat_table, ratebound_split, load_lxcat,
                     lxcat_collision_table, LXCatSet)
from .forcing import (HomogeneousField, DoubleLayerField, StepField, ConfinedDoubleLayerField, ElectromagneticField,
                      NullForcing, CombinedForcing, RK2Pusher, RestrictedForcing, RestrictedPusher, NullPusher)
from .population import (ElectronState, PhotonState, PositronState, ParticleArrays, Population, MultiPopulation,
                         init, advance, run, nparticles, nactives, weight, meanenergy, maxenergy, spread, posvar,
                         spectrum, repack, droplow, roulette, split, energy_table, ENERGY_TABLE_NODES,
                         kinenergy, AbstractCallback, VoidCallback, CombinedCallback,
                         CollisionCounter, PopulationTargetCallback, ParticleCountCallback, WallCallback,
                         RouletteCallback, SplitCallback)
from . import workloads, learned
from .learned import SamplerNet

co = constants
__version__ = "0.1.0"
