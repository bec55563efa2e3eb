"""Pure-Python ``numba.typed`` containers for the fixture shim."""


class List(list):
    @staticmethod
    def empty_list(*args, **kwargs):
        return List()


class Dict(dict):
    @staticmethod
    def empty(*args, **kwargs):
        return Dict()
