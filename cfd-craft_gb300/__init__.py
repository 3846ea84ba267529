"""GB300 pressure-projection engine for CFD-craft.

Modules:
  grid      -- Grid.build(case): the staggered grid arrays (crates/cfd-craft/src/grid.rs)
  pressure  -- project / solve_scaled / solve / apply / center_nullspaces (pressure.rs)
  engine    -- ctypes binding of libcfdgpu.so (include/cfdgpu.h)
  archive   -- run archives of device runs in the reference's format (output.rs write_run)
  sources   -- source density fields of a case's emissions (transport.rs source_fields)
  receptors -- receptor weights (transport.rs receptor_weights) for DeviceGrid.set_receptors
  synth     -- seeded synthetic cases of the benchmark configurations
  build     -- in-tree build of libcfdgpu.so for sm_103a
"""
from . import archive, engine, grid, pressure, receptors, sources, synth  # noqa: F401
