"""GB300-native compute core of the airbox-flow tool (parity voxelizer, fused
D3Q19 lattice-Boltzmann step, KPI reductions) behind the C ABI of
libairbox.so; ``engine`` mirrors the reference's src/engine.js surface."""
from .engine import (AirboxError, Geometry, Simulation, cpuStep, evaluate, makeFrame, parseSTL, prepare,  # noqa: F401
                     setupSim, simulate)
