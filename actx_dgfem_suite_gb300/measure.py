"""Array-context instantiation and queue synchronisation, mirroring
``actx_dgfem_suite/measure.py:16-55`` with a branch for the GB300 context."""

from __future__ import annotations

import gc

from actx_dgfem_suite_gb300.array_context import GB300DGArrayContext


def instantiate_actx_t(actx_t):
    """Construct an array context of type ``actx_t`` (``measure.py:16-45``);
    raises ``NotImplementedError`` for types this package does not provide."""
    gc.collect()
    if isinstance(actx_t, type) and issubclass(actx_t, GB300DGArrayContext):
        return actx_t()
    raise NotImplementedError(actx_t)


def finish_command_queue(actx) -> None:
    """Block until all work queued by ``actx`` is done (``measure.py:48-55``)."""
    if isinstance(actx, GB300DGArrayContext):
        actx.finish()
    else:
        raise NotImplementedError(type(actx))
