"""gbattract -- GB300-native docking energy/gradient path of gpuATTRACT 2.0.

The compute lives in libgbattract.so (CUDA for sm_103a, C ABI in
include/gbattract.h); this package holds the host-side mirror of the
reference's data model and request interface, the seeded synthetic workloads
and the build step.  Because the directory name is not a Python identifier the
package is imported under the name ``gbattract`` (see __graft_entry__.load_package).
"""
from .model import (DIELEC_CONSTANT, DIELEC_VARIABLE, FELEC, MODES_MAX, POTSHAPE_12_6,  # noqa: F401
                    POTSHAPE_8_6, GridOptions, GridSet, IntrplDesc, NLDesc, ParamTable, Protein,
                    attract_params, dofs_modes)
from . import synth  # noqa: F401


def build(verbose: bool = False):
    """Compiles libgbattract.so in-tree (sm_103a)."""
    from .build import build as _build
    return _build(verbose=verbose)


def __getattr__(name):
    # the device-facing API needs the compiled library; import it lazily so the
    # data model and generator stay usable while building
    if name in ("GbaContext", "GbaError"):
        from . import _lib, context
        return {"GbaContext": context.GbaContext, "GbaError": _lib.GbaError}[name]
    raise AttributeError(name)
