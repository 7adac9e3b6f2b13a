"""GB300-native (sm_103a) rebuild of LiveSpikeSorter's per-batch spike-sorting hot path.

The product is the C-ABI shared library built from ``csrc/`` (``liblss_gb300.so``):
preprocessing, template projection, the matching pursuit loop and PC-feature extraction
as hand-written CUDA, behind ``include/lss_gb300.h``.  ``sorter`` is the Python mirror of
that interface (ctypes); ``synth`` builds seeded recordings and ``oss_input/`` directories.
"""
__all__ = ["synth", "sorter"]
