"""GB300-native drop-in for the l3es pseudo-spectral DNS hot path.

Module names and function signatures mirror the reference package ``l3es``
(tumaer/ql-les-data): ``spectral_solver``, ``integrator``, ``utils``,
``init_fields``, ``combined``. Arrays are torch CUDA tensors (float32 fields,
complex64 spectra); the compute runs in the CUDA library behind ``_native``.
"""

__all__ = ["spectral_solver", "integrator", "utils", "init_fields", "combined"]
