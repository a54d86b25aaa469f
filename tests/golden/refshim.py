"""Import shim used only by ``make_golden.py`` to run the reference FEALPy here.

FEALPy imports plotting and mesh-IO packages (matplotlib, gmsh, vtk, pyevtk,
...) at class-definition time, e.g. ``fealpy/mesh/uniform_mesh_1d.py:509``.
None of them is used by the assemble/solve path, and none is installed in the
fixture-generation container, so this module registers a meta-path finder that
hands out inert stub modules for them.  Nothing in the product imports this.
"""
import importlib.abc
import importlib.machinery
import sys
import types

_STUB_ROOTS = ("matplotlib", "mpl_toolkits", "gmsh", "vtk", "vtkmodules",
               "pyevtk", "meshio", "ipdb", "pyvista", "OpenGL", "glfw")


class _Dummy:
    def __init__(self, *args, **kwargs):
        pass

    def __call__(self, *args, **kwargs):
        return _Dummy()

    def __getattr__(self, name):
        if name.startswith("__"):
            raise AttributeError(name)
        return _Dummy()

    def __mro_entries__(self, bases):
        return (object,)


class _StubModule(types.ModuleType):
    def __getattr__(self, name):
        if name.startswith("__"):
            raise AttributeError(name)
        return _Dummy


class _StubFinder(importlib.abc.MetaPathFinder, importlib.abc.Loader):
    def find_spec(self, fullname, path, target=None):
        if fullname.split(".")[0] in _STUB_ROOTS:
            return importlib.machinery.ModuleSpec(fullname, self, is_package=True)
        return None

    def create_module(self, spec):
        mod = _StubModule(spec.name)
        mod.__path__ = []
        return mod

    def exec_module(self, module):
        return None


def install(reference_root):
    """Install the stub finder and put ``reference_root`` first on sys.path."""
    if not any(isinstance(f, _StubFinder) for f in sys.meta_path):
        sys.meta_path.insert(0, _StubFinder())
    if reference_root not in sys.path:
        sys.path.insert(0, reference_root)
