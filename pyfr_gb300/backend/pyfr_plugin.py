"""Registration of the ``b200`` backend with PyFR itself.

PyFR picks its backend by name among the subclasses of
``pyfr.backends.base.BaseBackend`` (``pyfr/backends/__init__.py:10-11``,
``pyfr/__main__.py:237-240``).  Importing this module, where PyFR is
importable, defines that subclass: the b200 backend with PyFR's base
class behind it, so that ``get_backend('b200', cfg)``, ``pyfr -b b200
run`` and PyFR's own systems, integrators and plugins use it.  Everything
the backend interface needs is the b200 backend's own; PyFR's base class
only supplies what the b200 backend does not override.

A PyFR installation makes the backend selectable by importing this module
before ``pyfr.__main__.main()`` computes the ``-b`` choices (a launcher
that imports it, or a ``.pth`` file with ``import
pyfr_gb300.backend.pyfr_plugin``).
"""

from pyfr.backends.base import BaseBackend

from pyfr_gb300.backend.base import B200Backend


class B200PyFRBackend(B200Backend, BaseBackend):
    """The b200 backend as a PyFR backend class."""
    name = 'b200'

    def __init__(self, cfg):
        B200Backend.__init__(self, cfg)
