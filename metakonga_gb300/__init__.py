"""GB300-native DEM contact step for xdynamics (metakonga/metakonga).

The compute path is the CUDA library ``libxdem`` (metakonga_gb300/csrc), built
for sm_103a and reached through its C ABI (include/xdem.h).  This package holds
the host-side mirror of the reference's DEM interface (grid, integrator,
contact manager, simulation step) on top of that ABI, plus the synthetic scene
generators.  There is no CPU fallback: every compute call goes to the GPU.
"""
