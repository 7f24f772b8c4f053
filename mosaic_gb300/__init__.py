"""mosaic_gb300: the MOSAIC kinematic X-ray scattering sum, GB300-native.

The scattering entry point ``beam.atomic_scattering_kinematic`` takes the
reference's sample / detector / stage objects (or the ones here) and runs the
sum in hand-written sm_103a CUDA kernels behind the C ABI of
``libmosaic_kin.so`` (``include/mosaic_kin.h``).
"""
from .beam import beam
from .geometry import Detector, Stage, StaticStage, polarization_from_rate, polarization_state
from .sample import ChunkedSample, DiskSample, thermal_displacement, write_sample
from .tables import ScatteringTables

__all__ = ["beam", "Detector", "Stage", "StaticStage", "ChunkedSample", "DiskSample", "write_sample", "ScatteringTables",
           "polarization_from_rate", "polarization_state", "thermal_displacement"]
__version__ = "1.0.0"
