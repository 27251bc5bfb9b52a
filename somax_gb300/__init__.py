"""GB300-native (sm_103a) multilayer quasi-geostrophic time step, a drop-in below somax's
QG model API.  The compute path is libqgcore.so (hand-written CUDA, C ABI in
include/qgcore.h); this package is the Python host side that mirrors somax's classes."""

from .qg import (  # noqa: F401
    SSPRK3, BaroclinicQG, BaroclinicQGDiagnostics, BaroclinicQGParams, BaroclinicQGPhysConsts, BaroclinicQGState,
    BarotropicQG, BarotropicQGDiagnostics, BarotropicQGParams, BarotropicQGPhysConsts, BarotropicQGState, Euler, Heun,
    MemberSpec, Plan, QGDiagnostics, QGEnsemble, QGParams, SaveAt, Solution, SomaxModel, State, Tsit5,
)
from .reparameterized import MultilayerSW2DState, ReparameterizedQG, ReparamQGDiagnostics  # noqa: F401
from .swm import (  # noqa: F401
    MultilayerShallowWater2D, MultilayerSW2DDiagnostics, MultilayerSW2DParams, MultilayerSW2DPhysConsts,
    NonlinearShallowWater2D, NonlinearSW2DDiagnostics, NonlinearSW2DParams, NonlinearSW2DPhysConsts, NonlinearSW2DState,
)
from .transforms import ModalTransform, StratificationProfile  # noqa: F401
from .gfd_testcases import (  # noqa: F401
    baroclinic_instability_swm, barotropic_jet_instability, doublegyre_baroclinic_qg, doublegyre_qg,
    doublegyre_reparameterized_qg,
)
