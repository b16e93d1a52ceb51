"""aeroapps_gb300: GB300-native drop-in for AeroApps' aerosol-optics + VLIDORT
TOA-radiance hot path.

  mie.ChemMie / mie.get_aop_vector          Chem_Mie tables + VLIDORT_getAOPvector (FP32, GPU)
  vlidort.vlidort_scalar_lambert            VLIDORT_Scalar_Lambert (FP64, GPU)
  synth.make_columns                        seeded synthetic columns of the benchmark configs

All compute runs in libaerort.so (CUDA, sm_103a); there is no CPU fallback.
"""
from . import build  # noqa: F401

__all__ = ["build", "mie", "vlidort", "synth"]
