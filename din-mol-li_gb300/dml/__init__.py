"""Host-side mirror of din-mol-Li's hot-path routines over the GB300 C ABI."""
from ._abi import *  # noqa: F401,F403
