"""GB300-native (sm_103a) Factor Fields field evaluation and ray rendering.

Drop-in surface of autonomousvision/factor-fields' models/FactorFields.py and renderer.py for
basis_type = coeff_type = 'grid', running on hand-written CUDA kernels (libffgb.so) through a
C ABI (include/ff_native.h). No CPU fallback: the library must be built
(`python -m factor_fields_gb300.build`).
"""
from .config import Cfg, make_cfg, merged_cfg  # noqa: F401
from .field import FactorFields, MLPMixer, dct_dict  # noqa: F401

__all__ = ["Cfg", "make_cfg", "merged_cfg", "FactorFields", "MLPMixer", "dct_dict"]
