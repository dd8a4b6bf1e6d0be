"""GB300-native 3D space-charge kick with Ocelot's SpaceCharge plugin surface.

Drop-in use (replace Ocelot's import):

    from ocelot_gb300 import SpaceCharge
    sc = SpaceCharge(step=1, nmesh_xyz=[63, 63, 63])
    navi.add_physics_proc(sc, start, stop)   # Ocelot's Navigator, unchanged
"""
from .beam import DeviceParticleArray, ParticleArray
from .physics_proc import PhysProc
from .sc import Engine, SpaceCharge

__all__ = ["SpaceCharge", "PhysProc", "ParticleArray", "DeviceParticleArray", "Engine"]
__version__ = "0.1.0"
