import os


def get_pkg_data_filename(name, package=None):
    return os.path.join(package or '', name)
