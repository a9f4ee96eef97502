"""optifax_gb300: GB300 (sm_103a) chi(2) split-step crystal-pass propagator and
synchronously pumped OPO engine with OptiFax's solver interface.

The compute path is the CUDA library optifax_gb300/_lib/liboptifax.so (C ABI
in include/optifax.h); physics.py prepares the solver inputs on the host.
"""
__version__ = "0.1.0"
