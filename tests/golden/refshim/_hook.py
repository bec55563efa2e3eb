"""Import hook that loads the reference package from source with numba-only
array-type literals (``np.uint32[::1]`` and friends) replaced by ``None``.

numpy 2.x rejects those subscripts without numba; the rewrite happens in
memory, so the read-only reference tree is never modified.
"""
import importlib.abc
import importlib.machinery
import re
import sys

_PAT = re.compile(r"np\.(u?int\d+|float\d+|complex\d+|bool_)\[[^\]\n]*\]")


class _Loader(importlib.machinery.SourceFileLoader):
    def get_code(self, fullname):
        src = self.get_data(self.path).decode("utf-8")
        src = _PAT.sub("None", src)
        return compile(src, self.path, "exec", dont_inherit=True)


class _Finder(importlib.abc.MetaPathFinder):
    def find_spec(self, fullname, path, target=None):
        if not (fullname == "hiten" or fullname.startswith("hiten.")):
            return None
        spec = importlib.machinery.PathFinder.find_spec(fullname, path)
        if spec is None or not isinstance(spec.loader, importlib.machinery.SourceFileLoader):
            return spec
        spec.loader = _Loader(fullname, spec.origin)
        return spec


sys.meta_path.insert(0, _Finder())
