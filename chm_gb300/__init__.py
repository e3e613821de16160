"""GB300 (sm_103a) implementation of CHM's PBSM3D blowing-snow step.

The step runs in libpbsm3d_cuda (chm_gb300/csrc, C ABI in include/pbsm3d.h);
chm_gb300.pbsm3d mirrors CHM's module interface over it and chm_gb300.synth
generates the seeded synthetic meshes and forcing.
"""
