"""Time schemes: registers and stage sequence of core/timescheme.py.

``Timescheme(param, state)`` allocates the register states the reference allocates
(core/timescheme.py:92-101): RK3_SSP keeps ds0, ds1, ds2; LFAM3 keeps dstate,
stateb and state; EF keeps dstate. The stages themselves (EF :113-122, LFAM3
:125-177, RK3_SSP :180-221) run inside libnyles_gb300.so (nyles_model_forward).
"""
from . import variables as var

SCHEMES = ("EF", "LFAM3", "RK3_SSP")


class Timescheme(object):
    def __init__(self, param, state, model=None, arena=None):
        timestepping = param["timestepping"]
        if timestepping not in SCHEMES:
            raise ValueError("unknown time scheme " + repr(timestepping))
        self.timestepping = timestepping
        self.prognostic_scalars = state.get_prognostic_scalars()
        dtype = state.storage.dtype if state.storage is not None else None
        device = state.storage.device if state.storage is not None else "cpu"
        self.registers, self.storage = var.get_prognostic_registers(param, 3, dtype=dtype, device=device,
                                                                    arena=arena)
        self.dstate = self.registers[0]
        if timestepping == "LFAM3":
            self.stateb = self.registers[1]
            self.state = self.registers[2]
            self.first = True
        if timestepping == "RK3_SSP":
            self.ds0, self.ds1, self.ds2 = self.registers
        self._model = model

    def set(self, rhs, diagnose_var):
        self.rhs = rhs
        self.diagnose_var = diagnose_var

    def register_pointers(self):
        """3 * nprog device pointers, register-major (C ABI nyles_model_bind)."""
        return [s.data_ptr() for reg in self.registers for s in reg.scalars()]

    def forward(self, state, t, dt, **kwargs):
        if self._model is None:
            raise RuntimeError("time scheme not attached to a model")
        self._model._check_state(state)
        return self._model.forward(t, dt)
