"""The ``b200`` backend (GB300, sm_103a) of the flux-reconstruction RHS."""

from pyfr_gb300.backend.base import B200Backend, NotSuitableError


def get_backend(name, cfg):
    """Backend lookup by name, as ``pyfr/backends/__init__.py:10-11``."""
    if name.lower() != B200Backend.name:
        raise ValueError(f'Unknown backend {name!r}; this package provides '
                         f'{B200Backend.name!r}')
    return B200Backend(cfg)
