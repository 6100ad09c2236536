class ConfigItem:
    def __init__(self, default, description='', *args, **kwargs):
        self.default = default

    def __get__(self, obj, objtype=None):
        return self.default


class ConfigNamespace:
    pass
