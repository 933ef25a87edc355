"""h5py stand-in: importable, but any file access fails."""


class File(object):
    def __init__(self, *args, **kwargs):
        raise NotImplementedError("h5py is not available in this stand-in")
