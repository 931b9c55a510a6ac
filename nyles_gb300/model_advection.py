"""The pure advection model (the interface of the reference's core/model_advection.py).

``Advection(param, grid)`` advects the buoyancy b with the contravariant velocity U
stored in the state, which the model never changes: ``rhs`` is the tracer flux
divergence of b (core/model_advection.py:59-61, with its diffusion on the last stage
when diff_coef names b), ``diagnose_var`` fills the halo of b (:33-35), and
``make_u_divergentfree`` projects the covariant velocity u and sets U and div from it
(:38-53). The time schemes, graphs, snapshots and profiling are those of ``LES``.

Two defects of the reference are repaired, as their intent is plain: its constructor
calls ``Tracer_numerics`` without the `param` argument (TypeError), and
``make_u_divergentfree`` builds the superseded Python multigrid and calls
``compute_p`` without `ngbs`; here the projection is the one of LES.diagnose_var
(mgfor's multigrid, p = x*dx**2). ``update_stats`` records mean and standard deviation
of b (the reference's version calls an undefined numpy name and keeps nothing).
"""
from . import _native as nat
from .model_les import LES


class Advection(LES):
    modelname = "advection"

    def __init__(self, param, grid, device=None):
        if param.get("n_tracers", 0):
            raise ValueError("the advection model advects b only (core/model_advection.py:21); "
                             "set n_tracers = 0")
        super().__init__(param, grid, device=device)
        self.forced = False          # the reference's Advection has no forcing hook
        self.traclist = ["b"]
        self.order = param.get("orderA", 5)

    def make_u_divergentfree(self):
        """Project u (fill, multigrid, p = x*dx**2, u -= grad p), then U = u/dx**2 and
        div of U with its halo filled."""
        nat.check(self.lib.nyles_model_project(self._h, nat.stream_ptr()))

    def update_stats(self):
        b = self.state.b.view()
        self.stats.append({"bmean": float(b.mean()), "bstd": float(b.std(unbiased=False))})
