"""molmod.io stand-in."""


class XYZWriter(object):
    def __init__(self, fn, symbols):
        self.fn = fn

    def dump(self, title, pos):
        pass
