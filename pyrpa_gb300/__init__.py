"""GB300-native FLEX / RPA / linearized-Eliashberg engine for pyrpa.

``pyrpa_gb300.flibs`` mirrors the hot-path functions of pyrpa's ``libs.flibs``
on top of the CUDA library ``libfmod.so`` built from ``csrc/`` by
``pyrpa_gb300.build``; ``pyrpa_gb300.models`` builds the benchmark models.
"""
__all__ = ["flibs", "build", "models"]
