"""GB300-native eigensolver for planetary normal modes: the eigensolve path
of NormalModes (Chebyshev-filtered Lanczos on A x = lambda B x) behind the
C-ABI of include/nmgpu.h.

Modules: ``nmgpu`` (the GPU library: Solver, KPM slicing, adjoint),
``model`` (models, input and result files, FEM assembly), ``run`` (a
NormalModes job from its global_conf), ``timeop`` and ``compare``
(measurement), ``build`` (the native build).
"""
