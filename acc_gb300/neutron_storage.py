"""Neutron storage files (.mcv), the format of mcni's neutron_storage that the
reference reads in acc/components/sources/neutronfromstorage.py:58-61 and
that its tests ship (tests/components/sources/singletestneutron.mcv,
written by create_neutron_storage_for_test.py).

The layout, as those files hold it:

* a header of 1100 bytes: the text "Neutron", NUL-padded to 64 bytes, then
  the number of neutrons as a little-endian 64-bit integer at byte 64, then
  zeros;
* then the neutrons, 10 little-endian float64 each, in the order
  x y z vx vy vz sx sy t p (`ndblsperneutron`).

`storage(path, mode)` mirrors the calls the reference makes on mcni's
storage object: ``storage(path, 'r').read(asnpyarr=True, wrap=False)``,
``storage(path, 'w').write(neutrons)`` and ``close()``.  Neutrons are
(N, 10) float64 NumPy arrays here; there is no neutron_buffer type.
"""

import os
import struct

import numpy as np

ndblsperneutron = 10
MAGIC = b"Neutron"
HEADER_BYTES = 1100
COUNT_OFFSET = 64
ROW_BYTES = 8 * ndblsperneutron
_DTYPE = np.dtype("<f8")


def header(count):
    """The 1100-byte header of a file of `count` neutrons."""
    h = bytearray(HEADER_BYTES)
    h[:len(MAGIC)] = MAGIC
    h[COUNT_OFFSET:COUNT_OFFSET + 8] = struct.pack("<Q", int(count))
    return bytes(h)


def _read_header(f, path):
    h = f.read(HEADER_BYTES)
    if len(h) < HEADER_BYTES or h[:len(MAGIC) + 1] != MAGIC + b"\0":
        raise ValueError(f"{path}: not a neutron storage (.mcv) file")
    (count,) = struct.unpack_from("<Q", h, COUNT_OFFSET)
    return count


def as_rows(neutrons):
    """An (N, 10) float64 array of `neutrons` (any array of N x 10 values)."""
    a = np.ascontiguousarray(neutrons, dtype=np.float64)
    if a.size % ndblsperneutron:
        raise ValueError("neutrons must hold 10 values each "
                         "(x y z vx vy vz sx sy t p)")
    return a.reshape(-1, ndblsperneutron)


class storage:
    """A neutron storage file opened for reading ('r'), writing ('w', which
    truncates) or appending ('a')."""

    def __init__(self, path, mode="r"):
        if mode not in ("r", "w", "a"):
            raise ValueError("mode must be 'r', 'w' or 'a'")
        self.path, self.mode = str(path), mode
        if mode == "w" or (mode == "a" and not os.path.exists(self.path)):
            with open(self.path, "wb") as f:
                f.write(header(0))
            mode = "a"
        self._f = open(self.path, "rb" if mode == "r" else "r+b")
        self.count = _read_header(self._f, self.path)
        size = os.fstat(self._f.fileno()).st_size
        if size < HEADER_BYTES + self.count * ROW_BYTES:
            raise ValueError(f"{self.path}: header says {self.count} neutrons "
                             f"but the file holds "
                             f"{(size - HEADER_BYTES) // ROW_BYTES}")
        self._pos = 0

    def read(self, n=None, asnpyarr=True, wrap=True):
        """The next `n` neutrons (all that are left when n is None) as an
        (n, 10) array.  With `wrap`, reading past the last neutron goes on
        from the first; without, it stops at the last."""
        if self.mode != "r":
            raise IOError(f"{self.path}: not opened for reading")
        left = self.count - self._pos
        if n is None:
            n = left
        n = int(n)
        if n < 0:
            raise ValueError("cannot read a negative number of neutrons")
        if not wrap:
            n = min(n, left)
        out = np.empty((n, ndblsperneutron))
        done = 0
        while done < n:
            if self._pos == self.count:
                if not self.count:
                    raise ValueError(f"{self.path}: no neutrons to wrap over")
                self._pos = 0
            k = min(n - done, self.count - self._pos)
            self._f.seek(HEADER_BYTES + self._pos * ROW_BYTES)
            out[done:done + k] = np.frombuffer(
                self._f.read(k * ROW_BYTES), dtype=_DTYPE).reshape(k, -1)
            self._pos += k
            done += k
        return out

    def write(self, neutrons):
        """Append `neutrons` ((N, 10) values) and update the header's count."""
        if self.mode == "r":
            raise IOError(f"{self.path}: opened for reading")
        rows = as_rows(neutrons)
        self._f.seek(HEADER_BYTES + self.count * ROW_BYTES)
        self._f.write(rows.astype(_DTYPE, copy=False).tobytes())
        self.count += len(rows)
        self._f.seek(COUNT_OFFSET)
        self._f.write(struct.pack("<Q", self.count))
        self._f.flush()

    def close(self):
        if self._f is not None:
            self._f.close()
            self._f = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def load(path):
    """All neutrons of a storage file, (N, 10) float64."""
    with storage(path, "r") as s:
        return s.read(wrap=False)


def save(path, neutrons, append=False):
    """Write (or, with `append`, add) `neutrons` to a storage file."""
    with storage(path, "a" if append else "w") as s:
        s.write(neutrons)
