"""diffrax_gb300: GB300-native batched diffeqsolve.

A drop-in for ``jax.vmap(diffrax.diffeqsolve)`` over registered vector fields,
executed by hand-written sm_103a kernels in libgbdx.so (see include/gbdx.h).
"""
from ._core import (
    AbstractAdjoint, AbstractField, AbstractSolver, AbstractStepSizeController, AbstractTerm,
    BacksolveAdjoint, ClipStepSizeController, ConstantStepSize, ControlTerm, Dopri5, Dopri8, Euler, Heun, LotkaVolterra,
    MLPField, MultiTerm, ODETerm, OrnsteinUhlenbeck, TanhDiagonalDiffusion, PIDController, RecursiveCheckpointAdjoint,
    RESULTS, SaveAt, SubSaveAt, Solution, Tsit5, VanDerPol, VirtualBrownianTree, adjoint_rms_seminorm,
    rms_norm, Event, LinearCondition, Newton, SteadyStateCondition, steady_state_event,
    AbstractBrownianIncrement, BrownianIncrement, SEA, ShARK, SpaceTimeLevyArea, SRA1,
    AbstractProgressMeter, NoProgressMeter, TextProgressMeter, TqdmProgressMeter,
)
from ._integrate import DenseInterpolation, diffeqsolve, lower
from ._tune import GraphedSolve, autotune_launch, tuned_shapes
from . import distributed

__version__ = "0.1.0"


def build(force: bool = False) -> str:
    """Compile libgbdx.so for sm_103a (in-tree) and return its path."""
    from . import _build
    return _build.build(force=force)


def load_library():
    """Load libgbdx.so (building it when stale)."""
    from . import _lib
    return _lib.load()
