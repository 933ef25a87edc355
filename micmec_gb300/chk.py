"""Reader and writer for MicMec's text checkpoint (CHK) files.

The format is the one the reference reads with ``molmod.io.chk.load_chk`` and
writes with ``dump_chk`` (micmec/system.py:213-259, 298-316). Each field starts
with a header line ``<name padded to 40> kind=<kind> <shape or value>``, where
``kind`` is one of ``int``, ``flt``, ``str``, ``intar``, ``fltar``, ``bln``,
``blnar`` or ``none``. Scalars and strings sit on the header line. Arrays put
their comma-separated shape on the header line and their values, row-major,
four to a line, on the lines that follow (e.g. data/3x3x3_test_micmec.chk:1-60).
"""

import numpy as np

__all__ = ["load_chk", "dump_chk"]


def load_chk(fn):
    """Load a CHK file into a ``dict`` of NumPy arrays, numbers and strings."""
    result = {}
    with open(fn) as f:
        lines = f.read().splitlines()
    i = 0
    while i < len(lines):
        line = lines[i]
        i += 1
        if not line.strip():
            continue
        name = line[:40].strip()
        rest = line[40:].split(None, 1)
        if not rest or not rest[0].startswith("kind="):
            raise IOError("Malformed CHK header line: %r" % line)
        kind = rest[0][5:]
        tail = rest[1].strip() if len(rest) > 1 else ""
        if kind == "str":
            result[name] = tail
        elif kind == "int":
            result[name] = int(tail)
        elif kind == "flt":
            result[name] = float(tail)
        elif kind == "bln":
            result[name] = tail.strip().lower() in ("true", "1")
        elif kind == "none":
            result[name] = None
        elif kind in ("intar", "fltar", "blnar", "strar"):
            shape = tuple(int(s) for s in tail.split(",")) if tail else (0,)
            size = int(np.prod(shape)) if shape else 1
            words = []
            while len(words) < size:
                words.extend(lines[i].split())
                i += 1
            if kind == "intar":
                arr = np.array([int(w) for w in words[:size]], dtype=np.int64)
            elif kind == "fltar":
                arr = np.array([float(w) for w in words[:size]], dtype=np.float64)
            elif kind == "strar":  # right-aligned words without blanks (atom type names)
                arr = np.array(words[:size], dtype=object)
            else:
                arr = np.array([w.lower() in ("true", "1") for w in words[:size]])
            result[name] = arr.reshape(shape)
        else:
            raise IOError("Unknown CHK kind %r for field %r" % (kind, name))
    return result


def _fmt_float(x):
    return "% 22.15e" % x


def dump_chk(fn, data):
    """Write a ``dict`` to a CHK file in the layout :func:`load_chk` reads."""
    with open(fn, "w") as f:
        for key in sorted(data):
            value = data[key]
            head = "%-40s" % key
            if value is None:
                f.write(head + "kind=none\n")
            elif isinstance(value, str):
                f.write(head + "kind=str   %s\n" % value)
            elif isinstance(value, (bool, np.bool_)):
                f.write(head + "kind=bln   %s\n" % bool(value))
            elif isinstance(value, (int, np.integer)):
                f.write(head + "kind=int   %i\n" % value)
            elif isinstance(value, (float, np.floating)):
                f.write(head + "kind=flt   %s\n" % _fmt_float(value))
            else:
                arr = np.asarray(value)
                if arr.dtype.kind in "iu":
                    kind, fmt = "intar", lambda v: "%22i" % v
                elif arr.dtype.kind == "b":
                    kind, fmt = "blnar", lambda v: "%22s" % bool(v)
                else:
                    arr = arr.astype(np.float64)
                    kind, fmt = "fltar", _fmt_float
                shape = ",".join(str(s) for s in arr.shape)
                f.write(head + "kind=%s %s\n" % (kind, shape))
                flat = arr.ravel()
                for j in range(0, flat.size, 4):
                    f.write(" ".join(fmt(v) for v in flat[j:j + 4]) + "\n")
