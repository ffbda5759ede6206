"""GB300 (sm_103a) SSA/DIVA ice-velocity solver with Yelmo's solver interface."""
from .params import YdynParams  # noqa: F401
from . import abi, configs  # noqa: F401
