"""``SourceModule``-like objects for the drop-in modules.

The reference builds PyCUDA modules at run time and launches kernels as
``module.get_function(name)(*args, block=(bx, by, 1), grid=(gx, gy), shared=bytes)``
(``gtrap/geebls.py:10-22``, ``gtrap/gtls.py:11-27``, ``gtrap/gfilter.py:8-89``,
``gtrap/getstat.py:10-62``).  Here ``get_function`` returns a callable with the same
argument order that maps the launch configuration onto the native entry point
(e.g. ``grid[1]`` is the number of curves, ``block[0]`` the gtls width count).
"""
from __future__ import annotations


class KernelFunction:
    def __init__(self, name, impl):
        self.name = name
        self._impl = impl

    def __call__(self, *args, block=(1, 1, 1), grid=(1, 1), shared=0, stream=None, **kw):
        block = tuple(int(b) for b in block) + (1,) * (3 - len(block))
        grid = tuple(int(g) for g in grid) + (1,) * (2 - len(grid))
        return self._impl(*args, block=block, grid=grid, shared=int(shared), stream=stream, **kw)

    def __repr__(self):
        return "<gtrap_gb300 kernel %s>" % self.name


class Module:
    def __init__(self, functions: dict):
        self._functions = dict(functions)

    def get_function(self, name: str) -> KernelFunction:
        try:
            return KernelFunction(name, self._functions[name])
        except KeyError:
            raise LookupError("module has no kernel named %r (available: %s)"
                              % (name, ", ".join(sorted(self._functions)))) from None
