"""Iterations with recorded state and scheduled hooks.

An ``Iterative`` (an MD integrator or an optimiser) advances a counter. At every
counter value it runs the hooks scheduled for it; just before the first of them runs,
it refreshes its *recorded state*: a ``StateItem`` per quantity (energy, positions,
domain, ...) that reads the quantity from the iterative and keeps the value together
with its shape and dtype, from which trajectory writers size their datasets.

The public names, the state keys ("counter", "epot", "pos", "temp", "volume", "domain",
"epot_contribs", ...) and the hook schedule (a hook with ``start`` and ``step`` runs at
counters start, start + step, ...) are those of the reference's
micmec/sampling/iterative.py:42-222, which writers, hooks and user scripts rely on.
"""

import copy

import numpy as np

__all__ = [
    "Iterative", "StateItem", "AttributeStateItem", "PosStateItem", "EPotContribStateItem",
    "ConsErrStateItem", "TemperatureStateItem", "VolumeStateItem", "DomainStateItem", "Hook",
]


def _layout(value):
    """(shape, dtype) under which a recorded value is stored: arrays keep theirs, scalars are 0-d."""
    if isinstance(value, np.ndarray):
        return value.shape, value.dtype
    return (), type(value)


class StateItem(object):
    """One recorded quantity.

    ``reader(iterative)`` returns the current value; ``attrs(iterative)`` (optional) yields
    (name, value) metadata that a writer attaches to the quantity's dataset. Subclasses may
    override ``get_value`` / ``iter_attrs`` instead of passing functions.
    """

    def __init__(self, key, reader=None, attrs=None):
        self.key = key
        self._reader = reader
        self._attrs = attrs
        self.value = None
        self.shape = None
        self.dtype = None

    def get_value(self, iterative):
        if self._reader is None:
            raise NotImplementedError("StateItem %r has no reader" % self.key)
        return self._reader(iterative)

    def iter_attrs(self, iterative):
        return iter(()) if self._attrs is None else self._attrs(iterative)

    def update(self, iterative):
        self.value = self.get_value(iterative)
        if self.shape is None:  # the layout is fixed by the first value seen
            self.shape, self.dtype = _layout(self.value)

    def copy(self):
        """A fresh item of the same kind (no value, layout not yet known)."""
        clone = copy.copy(self)
        clone.value = clone.shape = clone.dtype = None
        return clone


class AttributeStateItem(StateItem):
    """The iterative's attribute of the same name (None while it does not exist)."""

    def __init__(self, key):
        StateItem.__init__(self, key, lambda it: getattr(it, key, None))


class PosStateItem(StateItem):
    def __init__(self):
        StateItem.__init__(self, "pos", lambda it: it.mmf.system.pos)


class TemperatureStateItem(StateItem):
    """Instantaneous temperature, stored with the degrees of freedom it was computed for."""

    def __init__(self):
        StateItem.__init__(self, "temp", lambda it: getattr(it, "temp", None), lambda it: iter([("ndof", it.ndof)]))


class VolumeStateItem(StateItem):
    def __init__(self):
        StateItem.__init__(self, "volume", lambda it: it.mmf.system.domain.volume)


class DomainStateItem(StateItem):
    def __init__(self):
        StateItem.__init__(self, "domain", lambda it: it.mmf.system.domain.rvecs)


class ConsErrStateItem(StateItem):
    """A statistic of the integrator's conserved-quantity tracker (None if it has no such field)."""

    def __init__(self, key):
        StateItem.__init__(self, key, lambda it: getattr(it._cons_err_tracker, key, None))


def _part_energies(iterative):
    return np.array([part.energy for part in iterative.mmf.parts])


def _part_names(iterative):
    yield "epot_contrib_names", np.array([part.name for part in iterative.mmf.parts], dtype="S")


class EPotContribStateItem(StateItem):
    """The energy of every part of the force field, with the parts' names as metadata."""

    def __init__(self):
        StateItem.__init__(self, "epot_contribs", _part_energies, _part_names)


class Hook(object):
    """A routine the iterative calls at counters ``start``, ``start + step``, ...

    ``modifies_state``: False for hooks that only read the iterative's state (writers,
    logs); the device MD paths then keep stepping while such a hook runs on a snapshot.
    """

    name = None
    kind = None
    method = None
    modifies_state = True

    def __init__(self, start=0, step=1):
        self.start = start
        self.step = step

    def expects_call(self, counter):
        offset = counter - self.start
        return offset >= 0 and offset % self.step == 0

    def __call__(self, iterative):
        raise NotImplementedError


def _hook_list(hooks):
    if hooks is None:
        return []
    if hasattr(hooks, "__len__"):
        return hooks  # the caller's list itself: hooks appended by the iterative show up there
    return [hooks]


class Iterative(object):
    """Counter, recorded state and hooks shared by the integrators and optimisers.

    ``default_state`` (class attribute) lists the items every instance records; ``state``
    adds more. ``propagate`` performs one iteration and returns True to stop early.
    """

    default_state = []
    log_name = "ITER"

    def __init__(self, mmf, state=None, hooks=None, counter0=0):
        self.mmf = mmf
        self.state_list = [item.copy() for item in self.default_state] + list(state or [])
        self.state = {item.key: item for item in self.state_list}
        self.hooks = _hook_list(hooks)
        self._add_default_hooks()
        self.counter0 = counter0
        self.counter = counter0
        self.initialize()

    def _add_default_hooks(self):
        """Subclasses append the hooks they always want (e.g. a screen log)."""

    def initialize(self):
        self.call_hooks()

    def call_hooks(self):
        """Run the hooks scheduled for the current counter, on freshly recorded state."""
        due = [hook for hook in self.hooks if hook.expects_call(self.counter)]
        if not due:
            return
        for item in self.state_list:
            item.update(self)
        for hook in due:
            hook(self)

    def run(self, nsteps=None):
        """Iterate ``nsteps`` times, or until ``propagate`` asks to stop (nsteps None: only then)."""
        done = 0
        while nsteps is None or done < nsteps:
            done += 1
            if self.propagate():
                break
        self.finalize()

    def propagate(self):
        self.counter += 1
        self.call_hooks()

    def finalize(self):
        pass
