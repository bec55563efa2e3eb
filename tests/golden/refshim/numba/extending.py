from numba import _decorator as overload, _decorator as register_jitable  # noqa: F401
