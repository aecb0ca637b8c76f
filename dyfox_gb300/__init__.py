"""dyfox_gb300: the GB300 (sm_103a) diffraction hot path of DYFOX.

Drop-in modules (same call signatures as DYFOX):

    dyfox_gb300.laue          solve_dislocation, solve_pristine, LaueGrid
    dyfox_gb300.dislocations  compute_H_grid, H_plane, segment helpers
    dyfox_gb300.bragg         solve_surface_batch, solve_bragg_stable,
                              perfect_symbol, BraggConfig
    dyfox_gb300.backend       FP64, FP32, to_numpy, free_gpu
    dyfox_gb300.crystal       DIAMOND, CrystalParams
    dyfox_gb300.units         deviation_from_urad, ...
    dyfox_gb300.optics        Optics, image_intensity, apply_pupils
    dyfox_gb300.rocking       com_maps, planewave_rocking
    dyfox_gb300.cache         WaveCache (DYFOX's cache keys and files)
    dyfox_gb300.illumination  condenser and energy-band quadrature nodes

Additions with no DYFOX counterpart:

    dyfox_gb300.batch         Batch: uneven Laue and Bragg instances in one
                              CUDA graph
    dyfox_gb300.autotune      launch-shape tuner of the Laue march
    dyfox_gb300.learned       U-Net shooting guess for the Bragg solve
    dyfox_gb300.workloads     the seeded benchmark configurations

Compute runs in libdyfox_gb300.so (hand-written CUDA for sm_103a, C ABI in
include/dyfox_gb300.h); importing the package does not touch the GPU.
"""

__version__ = "0.1.0"
