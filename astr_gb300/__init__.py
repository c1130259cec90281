"""GB300-native (sm_103a) right-hand-side hot path of the ASTR compressible
Navier-Stokes solver: compact derivatives, compact filter, convective and
viscous residuals, primitive recovery and the RK3 stage update, behind the C
ABI of ``include/astr_gpu.h``."""

__all__ = ["capi", "solver", "build_ext"]
