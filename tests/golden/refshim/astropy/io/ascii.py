def read(*args, **kwargs):
    raise NotImplementedError('ascii.read is not provided by the test shim')
