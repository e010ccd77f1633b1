"""pelelm_gb300: GB300-native (sm_103a) replacement of the PelePhysics chemistry reactor
that PeleLM's advance_chemistry drives (Source/PeleLM.cpp:5626-5845).

The product is the native library ``libpelelm_gb300.so`` (C ABI: include/pelelm_gb300.h);
``pelelm_gb300.reactor`` mirrors the reference's ReactorBase interface over it for Python
callers, and ``pelelm_gb300.workloads`` builds the seeded synthetic benchmark inputs.
"""
__all__ = ["reactor", "workloads", "mech"]
