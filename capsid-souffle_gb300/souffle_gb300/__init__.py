"""GB300-native force-and-integrate path for SOUFFLE capsid simulations.

Python side: geometry and state generators in the reference's file formats, and
a ctypes binding to the C-ABI library ``libsouffle_gb300.so``.
"""
