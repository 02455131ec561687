"""
GB300-native tubular segmentation: Frangi vesselness, direction sign
adjustment, gradient vector flow and continuous max-flow with anisotropic TV,
as hand-written sm_103a CUDA kernels behind a C ABI
(include/miccai2016_gb300.h).

The drop-in modules keep the Python call surface of the reference's
processing modules: continuous_cut_anisotropic_gpu (CmfCutQAnisotropicGpu).
"""
__version__ = "0.1.0"
