"""GB300-native implementation of CABLE's per-timestep tile physics (the
offline ``cbm()`` call): radiation, canopy energy balance with coupled
photosynthesis / stomatal conductance, and soil / snow heat and water, one
GPU thread per tile.  See ``include/cablegpu.h`` for the C ABI."""
from . import workloads  # noqa: F401

__all__ = ["workloads", "runtime", "build"]
