"""GB300-native batched cycle simulation for RRTL designs.

Package layout:
  builder   -- RTL design builder emitting the design interchange JSON
  netlist   -- Yosys JSON gate-netlist importer
  workloads -- seeded synthetic designs and job streams
  sim       -- GpuBatchSimulator over the C ABI (librrtl_gb300.so)
  build     -- in-tree build of the CUDA/C++ library
"""
from .builder import Design, concat, lit, lit_s, lit_u, mem_read, mux, sint, uint  # noqa: F401
