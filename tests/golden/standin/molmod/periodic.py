"""molmod.periodic stand-in (only ``periodic[55].symbol`` is used by the reference)."""


class _Elem(object):
    symbol = "Cs"


class _Periodic(object):
    def __getitem__(self, key):
        return _Elem()


periodic = _Periodic()
