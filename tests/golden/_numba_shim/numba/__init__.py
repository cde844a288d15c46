"""Inert stand-in for numba, used only to run pytreegrav's own Python source as plain Python.

numba is not installed in this environment, but every pytreegrav module imports it at module
scope. This package makes the decorators identity functions, ``prange`` the builtin ``range``,
type objects callable/subscriptable placeholders, ``get_num_threads()`` 1 and
``parallel_chunksize`` a no-op context, so the reference's unmodified algorithm runs (slowly) in
the interpreter. It is loaded solely by ``tests/golden/make_golden.py`` to generate fixtures;
nothing in the package or the tests imports it.
"""

import contextlib


def _decorator(*args, **kwargs):
    # bare use (@njit) or functional use (njit(f, fastmath=True, parallel=...))
    if len(args) == 1 and callable(args[0]) and not isinstance(args[0], (_Type, list)):
        return args[0]

    # parameterised use: @njit(...), @njit(sig, fastmath=True), @njit([sig]) ...
    def wrap(f):
        return f

    return wrap


njit = _decorator
jit = _decorator
vectorize = _decorator
guvectorize = _decorator
generated_jit = _decorator


def prange(*args):
    return range(*args)


def get_num_threads():
    return 1


def set_num_threads(n):
    return None


def get_parallel_chunksize():
    return 0


@contextlib.contextmanager
def parallel_chunksize(n):
    yield


class _Type:
    """Placeholder for numba scalar/array types: callable (signatures) and subscriptable."""

    def __init__(self, name):
        self.name = name

    def __call__(self, *args, **kwargs):
        return self

    def __getitem__(self, item):
        return self

    def __repr__(self):
        return f"<shim type {self.name}>"


float64 = _Type("float64")
float32 = _Type("float32")
int64 = _Type("int64")
int32 = _Type("int32")
boolean = _Type("boolean")
void = _Type("void")
uint64 = _Type("uint64")


def deferred_type():
    return _Type("deferred")


def optional(t):
    return t


class _Types:
    def __getattr__(self, name):
        return _Type(name)


types = _Types()
