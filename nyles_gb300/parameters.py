"""User parameters of a Nyles experiment.

Same interface and error behaviour as the reference's core/parameters.py:54-303:
one dictionary per category (model, physics, IO, animation, time, discretization,
MPI, multigrid) filled from ``defaults.json``; values can be changed but no key can be
added; ``check()`` raises :class:`UserParameterError` with the reference's messages;
``freeze()`` forbids any later change (for every instance, as in the reference).

GPU-specific settings live in a separate category ``gpu`` loaded from
``gpu_defaults.json`` (precision, multigrid tolerance/iterations/damping), so that the
reference parameter set stays unchanged.
"""
import datetime
import json
import os

CATEGORIES = ["model", "physics", "IO", "animation", "time", "discretization", "MPI", "multigrid"]
GPU_CATEGORY = "gpu"
ATTRIBUTES = ["type", "default", "avail", "doc"]


class UserParameterError(Exception):
    """An error occured with the user-set parameters."""


class DefaultsFileError(Exception):
    """An error occured in the file of default values."""

    def __init__(self, defaults_file, arg):
        super().__init__("bad format of file {}: {}".format(defaults_file, arg))


class InextensibleDict(dict):
    """dict whose keys are fixed at creation; ``freeze()`` also fixes the values.

    The frozen flag is shared by every instance (core/parameters.py:12-41).
    """

    frozen = False

    @classmethod
    def freeze(cls):
        cls.frozen = True

    @classmethod
    def unfreeze(cls):
        """Allow changes again (for several experiments in one process)."""
        cls.frozen = False

    def __setitem__(self, key, item):
        if InextensibleDict.frozen:
            raise UserParameterError("not possible to modify parameters after the creation of Nyles.")
        if key not in self:
            raise UserParameterError("not possible to add new key {!r} to the parameters.".format(key))
        dict.__setitem__(self, key, item)


_HERE = os.path.dirname(os.path.abspath(__file__))


class UserParameters(object):
    """Experiment parameters, one attribute (an InextensibleDict) per category."""

    DEFAULTS_FILE = "defaults.json"
    GPU_DEFAULTS_FILE = "gpu_defaults.json"
    TYPES = {
        "str": str,
        "int": int,
        "float": (float, int),
        "bool": bool,
        "dict": dict,
        "list or string": (list, tuple, str),
    }

    def __init__(self):
        with open(os.path.join(_HERE, self.DEFAULTS_FILE)) as f:
            defaults = json.load(f)
        self.check_defaults(defaults)
        with open(os.path.join(_HERE, self.GPU_DEFAULTS_FILE)) as f:
            gpu = json.load(f)
        self.documentations, self.options, self.types = {}, {}, {}
        for table in (defaults, gpu):
            for cat, params in table.items():
                values = {}
                for name, attrs in params.items():
                    values[name] = attrs["default"]
                    self.documentations[name] = attrs["doc"]
                    self.options[name] = attrs["avail"]
                    self.types[name] = attrs["type"]
                # a fresh copy of mutable defaults such as diff_coef = {}
                values = {k: (dict(v) if isinstance(v, dict) else v) for k, v in values.items()}
                # the frozen flag must not block the construction itself
                d = InextensibleDict()
                for k, v in values.items():
                    dict.__setitem__(d, k, v)
                setattr(self, cat, d)

    def help(self, parameter):
        if parameter in self.documentations:
            return self.documentations[parameter]
        raise ValueError("invalid parameter: {!r}".format(parameter))

    def possible_values(self, parameter):
        if parameter in self.options:
            return self.options[parameter]
        raise ValueError("invalid parameter: {!r}".format(parameter))

    def view_parameters(self):
        """All parameters in one (read-only by convention) dictionary."""
        out = {}
        for cat in CATEGORIES + [GPU_CATEGORY]:
            out.update(getattr(self, cat))
        return out

    def _check_value(self, parameter, value, powers_of_2):
        param_type = self.types[parameter]
        if not isinstance(value, self.TYPES[param_type]):
            raise UserParameterError("parameter {} must be {} {}, not {}".format(
                parameter, "an" if param_type == "int" else "a", param_type, type(value)))
        options = self.options[parameter]
        if isinstance(options, list):
            if value not in options:
                raise UserParameterError("parameter {} must be one of {}, not {!r}".format(parameter, options, value))
        elif options == "any":
            pass
        elif options == "> 0.0":
            if not value > 0.0:
                raise UserParameterError("parameter {} must be positive".format(parameter))
        elif options in (">= 0.0", ">= 0"):
            if not value >= 0.0:
                raise UserParameterError("parameter {} must be non-negative".format(parameter))
        elif options == ">= 1":
            if not value >= 1:
                raise UserParameterError("parameter {} must be at least 1".format(parameter))
        elif options == "2^n":
            if value not in powers_of_2:
                if value < max(powers_of_2):
                    raise UserParameterError("parameter {} must be a power of 2".format(parameter))
                raise UserParameterError(
                    "parameter {} is very large; if you are sure to use it, extend the variable "
                    "POWERS_OF_2 in this class to include your value".format(parameter))
        elif options == "[3 *] 2^n":
            if value not in powers_of_2 and value / 3 not in powers_of_2:
                if value < max(powers_of_2):
                    raise UserParameterError(
                        "parameter {} must be a power of 2 or 3 times a power of 2".format(parameter))
                raise UserParameterError(
                    "parameter {} is very large; if you are sure to use it, extend the variable "
                    "POWERS_OF_2 in this class to include your value".format(parameter))
        elif options == "any valid filename":
            if "/" in value:
                raise UserParameterError('parameter {} must not contain a "/"'.format(parameter))
        elif parameter == "variables_in_history":
            if not isinstance(value, (list, tuple)) and value not in ["all", "prognostic", "p+p"]:
                # argument order as in the reference message
                raise UserParameterError("value {!r} of parameter {} not understood".format(parameter, value))
        elif parameter == "datadir":
            pass

    def check(self):
        """Raise UserParameterError if any value is wrong (core/parameters.py:149-247)."""
        # the reference accepts powers of two up to 2**(year-2001)
        powers_of_2 = [2 ** n for n in range(datetime.datetime.now().year - 2000)]
        for parameter, value in self.view_parameters().items():
            self._check_value(parameter, value, powers_of_2)
        for x in "xyz":
            if self.MPI["np" + x] > self.discretization["global_n" + x]:
                raise UserParameterError("parameter np{} cannot be larger than global_n{}".format(x, x))

    @classmethod
    def check_defaults(cls, defaults):
        for category in CATEGORIES:
            if category not in defaults:
                raise DefaultsFileError(cls.DEFAULTS_FILE, "category {} missing".format(category))
        seen = []
        for category in defaults:
            if category not in CATEGORIES:
                raise DefaultsFileError(cls.DEFAULTS_FILE, "unknown category {}".format(category))
            for parameter, attributes in defaults[category].items():
                if parameter in seen:
                    raise DefaultsFileError(cls.DEFAULTS_FILE, "parameter {} appears twice".format(parameter))
                seen.append(parameter)
                for attribute in ATTRIBUTES:
                    if attribute not in attributes:
                        raise DefaultsFileError(cls.DEFAULTS_FILE,
                                                "attribute {} missing for parameter {}".format(attribute, parameter))
                for attribute in attributes:
                    if attribute not in ATTRIBUTES:
                        raise DefaultsFileError(cls.DEFAULTS_FILE,
                                                "unknown attribute {} for parameter {}".format(attribute, parameter))
                if attributes["type"] not in cls.TYPES:
                    raise DefaultsFileError(cls.DEFAULTS_FILE,
                                            "unknown type {} of parameter {}".format(attributes["type"], parameter))

    def freeze(self):
        InextensibleDict.freeze()
