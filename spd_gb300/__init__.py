"""GB300-native (sm_103a, FP64) SD-ADER step for the compressible Euler
equations, a drop-in for jpalafou/spd's SDADER_Simulator time step."""
from .simulator import FV_Simulator, SDADER_Simulator, SD_Simulator, Simulator  # noqa: F401
from .ensemble import SDADER_Ensemble  # noqa: F401
from . import initial_conditions  # noqa: F401

__all__ = ["Simulator", "SD_Simulator", "FV_Simulator", "SDADER_Simulator", "SDADER_Ensemble", "initial_conditions"]
