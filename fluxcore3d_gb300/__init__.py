"""fluxcore3d_gb300 -- GB300-native (sm_103a) conjugate-heat-transfer hot path.

Drop-in modules with the call surface of the reference solver package:
    fluxcore3d_gb300.solver.lbm_cuda_ext     (solver/lbm_cuda_ext.py)
    fluxcore3d_gb300.solver.mg_cuda_ext      (solver/mg_cuda_ext.py)
    fluxcore3d_gb300.solver.thermal_cuda_ext (solver/thermal_cuda_ext.py)
    fluxcore3d_gb300.solver.nlevel_mg_cuda   (solver/nlevel_mg_cuda.py)
    fluxcore3d_gb300.solver.mg_pcg           (solver/mg_pcg.py)
All compute runs in libfluxcore3d_gb300.so through its C ABI
(include/fluxcore3d_gb300.h).
"""
__version__ = "0.1.0"
