"""Argument validation helpers with the reference's behaviour
(pyop2/utils.py:49-233)."""
import functools
import inspect

import numpy as np

from pyop2_gb300.configuration import configuration
from pyop2_gb300.exceptions import DataTypeError, DataValueError

cached_property = functools.cached_property


def as_tuple(item, type=None, length=None, allow_none=False):
    """Coerce item to a tuple; check length and element types under type_check."""
    if item is None:
        t = ()
    else:
        try:
            t = tuple(item)
        except (TypeError, NotImplementedError):
            t = (item,) * (length or 1)
    if configuration["type_check"]:
        if length and not len(t) == length:
            raise ValueError("Tuple needs to be of length %d" % length)
        if type is not None:
            ok = all(isinstance(i, type) or (allow_none and i is None) for i in t)
            if not ok:
                raise TypeError("Items need to be of type %s" % (type,))
    return t


def tuplify(xs):
    """Turn a nested sequence into nested tuples."""
    try:
        return tuple(tuplify(x) for x in xs)
    except TypeError:
        return xs


def verify_reshape(data, dtype, shape, allow_none=False):
    """Convert data to an array of dtype with the given shape (in place
    reshape, so non-contiguous inputs fail), with the reference's errors."""
    try:
        t = np.dtype(dtype) if dtype is not None else None
    except TypeError:
        raise DataTypeError("Invalid data type: %s" % dtype)
    if data is None:
        if allow_none:
            return np.asarray([], dtype=t)
        raise DataValueError("Invalid data: None is not allowed!")
    try:
        a = np.asarray(data, dtype=t)
    except ValueError:
        raise DataValueError("Invalid data: cannot convert to %s!" % dtype)
    except TypeError:
        raise DataTypeError("Invalid data type: %s" % dtype)
    try:
        a = a.reshape(shape) if a.size == int(np.prod(shape)) else None
    except ValueError:
        a = None
    if a is None:
        raise DataValueError("Invalid data: expected %d values, got %d!" %
                             (np.prod(shape), np.asarray(data).size))
    return np.ascontiguousarray(a)


class _Validator:
    """Decorator base: checks named arguments when type_check is on."""

    def __init__(self, *checks):
        self.checks = checks

    def __call__(self, f):
        sig = inspect.signature(f)
        params = list(sig.parameters.values())
        # (name, position, default, check args) resolved once, not per call
        plan = []
        for name, *rest in self.checks:
            if name not in sig.parameters:
                continue
            pos = next(i for i, p in enumerate(params) if p.name == name)
            default = sig.parameters[name].default
            plan.append((name, pos, default, rest))

        @functools.wraps(f)
        def wrapper(*args, **kwargs):
            if configuration["type_check"]:
                for name, pos, default, rest in plan:
                    if pos < len(args):
                        value = args[pos]
                    elif name in kwargs:
                        value = kwargs[name]
                    elif default is not inspect.Parameter.empty:
                        value = default
                    else:
                        continue
                    self.check(name, value, *rest)
            return f(*args, **kwargs)
        return wrapper


class validate_type(_Validator):
    """validate_type(('name', types, exception), ...): None always passes."""

    def check(self, name, value, types, exception):
        if value is not None and not isinstance(value, types):
            raise exception("%s must be of type %s, not %s" % (name, types, type(value)))


class validate_in(_Validator):
    """validate_in(('name', allowed_values, exception), ...)."""

    def check(self, name, value, allowed, exception):
        if value not in allowed:
            raise exception("%s must be one of %s, not %r" % (name, allowed, value))


class validate_dtype(_Validator):
    """validate_dtype(('name', None, exception)): must be a numpy dtype or None."""

    def check(self, name, value, _unused, exception):
        if value is None:
            return
        try:
            np.dtype(value)
        except TypeError:
            raise exception("%s must be a valid dtype" % name)
