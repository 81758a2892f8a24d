"""obgc — GB300-native OceanBioME tracer-tendency engine (Python side of the C ABI).

The names mirror OceanBioME.jl's public API for the tracer-tendency path (the `!` of mutating
functions dropped): LOBSTER / NPZD and their components, the biogeochemistry plugin functions,
TwoBand / MultiBand / Prescribed light, CarbonChemistry, BoxModel, and an Oceananigans-style
NonhydrostaticModel with set_, time_step and update_biogeochemical_state.  Every computation runs in
libobgc.so (CUDA, sm_103a); importing works without it, calling does not.
"""
from . import _abi
from .box import BoxModel
from .forcing import Forcing
from .gas import (CarbonDioxideConcentration, CarbonDioxideGasExchangeBoundaryCondition, GasExchange,
                  OxygenGasExchangeBoundaryCondition)
from .pisces import PISCES, PiscesModel
from .columns import ColumnEngine
from .service import ColumnService
from .carbon import CarbonChemistry
from .grid import BoxModelGrid, RectilinearGrid
from .light import (MultiBandPhotosyntheticallyActiveRadiation, PrescribedPhotosyntheticallyActiveRadiation,
                    TwoBandPhotosyntheticallyActiveRadiation, default_surface_PAR, euphotic_depth)
from .model3d import (Clock, ExplicitTimeDiscretization, HorizontalScalarDiffusivity, NonhydrostaticModel,
                      ScalarDiffusivity, VerticallyImplicitTimeDiscretization, VerticalScalarDiffusivity,
                      compute_tendencies, set_, time_step, update_biogeochemical_state)
from .negatives import ScaleNegativeTracers, ZeroNegativeTracers
from .sediments import InstantRemineralisationSediment, SimpleMultiGSediment
from .distributed import PiscesSlabModel, SlabDecomposition, SlabModel, gather_runs, shard_runs
from .models import (LOBSTER, NPZD, CarbonateSystem, Detritus, NitrateAmmonia, NitrateAmmoniaIron, Nutrient,
                     NutrientsPlanktonDetritus, Oxygen, PhytoZoo, TwoParticleAndDissolved, VariableRedfieldDetritus,
                     biogeochemical_drift_velocity, conserved_tracers, eval_point, preset,
                     required_biogeochemical_auxiliary_fields, required_biogeochemical_tracers)
from .synthetic import (lobster_column_request, lobster_initial_conditions, mixed_layer_diffusivity,
                        pisces_initial_conditions,
                        npzd_column_ensemble, npzd_front_initial_conditions, random_streamfunction_velocity)

__all__ = [n for n in dir() if not n.startswith("_")]
