import inspect
import os


def get_pkg_data_filename(name, package=None):
    """Path of ``name`` relative to the calling module's directory (or
    ``package``'s), as astropy resolves package data."""
    if package is None:
        caller = inspect.stack()[1].filename
        base = os.path.dirname(os.path.abspath(caller))
    else:
        import importlib
        base = os.path.dirname(importlib.import_module(package).__file__)
    return os.path.join(base, name)
