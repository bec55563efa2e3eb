"""Register permissive stand-ins for the plotting/IO modules that the
reference imports at module level but that the propagation path never
calls (matplotlib, mpl_toolkits, pandas, h5py)."""
import importlib.abc
import importlib.machinery
import sys
import types

_PREFIXES = ("matplotlib", "mpl_toolkits", "pandas", "h5py")


class _Callable:
    def __call__(self, *a, **k):
        return _Callable()

    def __getattr__(self, name):
        if name.startswith("__"):
            raise AttributeError(name)
        return _Callable()

    def __iter__(self):
        return iter(())

    def __mro_entries__(self, bases):
        return (object,)


class _Permissive(types.ModuleType):
    def __getattr__(self, name):
        if name.startswith("__"):
            raise AttributeError(name)
        return _Callable()


class _StubLoader(importlib.abc.Loader):
    def create_module(self, spec):
        mod = _Permissive(spec.name)
        mod.__path__ = []
        return mod

    def exec_module(self, module):
        return None


class _StubFinder(importlib.abc.MetaPathFinder):
    def find_spec(self, fullname, path, target=None):
        if fullname.split(".")[0] in _PREFIXES:
            return importlib.machinery.ModuleSpec(fullname, _StubLoader(), is_package=True)
        return None


sys.meta_path.insert(0, _StubFinder())
