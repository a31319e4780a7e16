"""GB300-native PyHermes field pipeline.

Drop-in for the reference calls SFCProjection(params).run(), WindowFunc,
``field @ window``, Corr_2PCF and Corr_3PCF_Multipole; the hot loops run as
hand-written sm_103a CUDA kernels in libhermes_gb300.so (see include/).
"""

__version__ = "0.1.0"
