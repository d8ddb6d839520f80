"""``jax.sharding`` (test infrastructure; see ``jax/__init__.py``): one CPU
device, so a mesh only records its arguments."""


class Mesh:
    def __init__(self, devices, axis_names=()):
        self.devices = devices
        self.axis_names = tuple(axis_names)
