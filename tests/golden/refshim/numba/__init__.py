"""Pass-through stand-in for numba, used only to run the reference package
in pure-Python mode when generating golden fixtures (numba is not installed).

``njit``/``jit`` return the decorated function unchanged, so the reference's
kernels run as ordinary Python/numpy code with unchanged arithmetic order.
"""


class _Anything:
    """Object whose attributes, calls and subscripts all return itself."""

    def __getattr__(self, name):
        return self

    def __call__(self, *args, **kwargs):
        return self

    def __getitem__(self, item):
        return self


types = _Anything()
float64 = types
int64 = types
boolean = types
config = types


def _decorator(*args, **kwargs):
    if len(args) == 1 and callable(args[0]) and not kwargs:
        return args[0]

    def wrap(fn):
        return fn

    return wrap


njit = _decorator
jit = _decorator
vectorize = _decorator
guvectorize = _decorator
generated_jit = _decorator
prange = range


def get_num_threads():
    return 1


def set_num_threads(n):
    return None


def get_thread_id():
    return 0


def literal_unroll(x):
    return x


class _Extending:
    @staticmethod
    def overload(*a, **k):
        return _decorator

    @staticmethod
    def register_jitable(*a, **k):
        return _decorator(*a, **k)


extending = _Extending()
