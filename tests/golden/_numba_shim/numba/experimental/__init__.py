"""Inert stand-in for ``numba.experimental``: ``jitclass(spec)`` returns the class unchanged."""


def jitclass(spec=None, *args, **kwargs):
    if isinstance(spec, type):
        return spec

    def wrap(cls):
        return cls

    return wrap
