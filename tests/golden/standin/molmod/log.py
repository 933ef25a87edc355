"""molmod.log stand-in: a silent ScreenLog and a no-op TimerGroup."""
import contextlib


class TimerGroup(object):
    @contextlib.contextmanager
    def section(self, label):
        yield


class ScreenLog(object):
    do_warning = False
    do_medium = False
    do_high = False
    do_debug = False

    def __init__(self, *args, **kwargs):
        pass

    def __call__(self, *args, **kwargs):
        pass

    @contextlib.contextmanager
    def section(self, label):
        yield

    def hline(self, *a, **k):
        pass

    def blank(self, *a, **k):
        pass

    def warn(self, *a, **k):
        pass

    def print_footer(self):
        pass

    def set_level(self, level):
        pass
