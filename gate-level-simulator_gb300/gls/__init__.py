"""gls: GB300-native simulate stage of an SDF-annotated gate-level simulator.

Python side of the package: the synthetic workload generator, the netlist /
stimulus containers, and the ctypes binding of libgls (include/gls.h).
The simulation itself runs only in libgls's CUDA kernels.
"""
from .netlist import Netlist, Stimulus, V0, V1, VX, VZ  # noqa: F401
