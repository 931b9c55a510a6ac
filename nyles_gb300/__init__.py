"""nyles_gb300 — the Nyles LES time step on one GB300 GPU (sm_103a).

Drop-in for the reference's entry points:
    from nyles_gb300 import parameters, nyles
    param = parameters.UserParameters(); ...; n = nyles.Nyles(param); n.run()
The compute path is libnyles_gb300.so (C ABI in include/nyles_gb300.h).
"""
__version__ = "0.1.0"

__all__ = ["parameters", "topology", "variables", "grid", "timescheme", "model_les", "nyles", "multigrid",
           "serving"]
