"""quack_gb300 -- GB300-native restricted G0W0 / evGW (QuAcK's RG0W0 / evRGW call chain).

The compute lives in libqkgw.so (hand-written sm_103a CUDA, C ABI in include/qkgw.h);
``quack_gb300.api`` mirrors the reference's Fortran subroutines on top of it.
"""
__all__ = ["api", "synth", "build"]
