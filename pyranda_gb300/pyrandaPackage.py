"""Base class of the physics packages (pyranda/pyrandaPackage.py)."""


class pyrandaPackage:
    def __init__(self, name, pysim):
        self.name = name
        self.pyranda = pysim
        self.sMap = {}

    def get_sMap(self):
        self.sMap = {}
