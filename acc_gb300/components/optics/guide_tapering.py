"""Segmented tapered guide (acc/components/optics/guide_tapering.py:22-291):
equal-length segments, each a four-mirror channel tapering from w1 x h1 to
w2 x h2, with separate supermirror coatings for the side (mx, Qcx, alphax)
and top/bottom (my, Qcy, alphay) mirror pairs."""

import numpy as np

from ... import _native as nat
from ..ComponentBase import ComponentBase, set_param

category = 'optics'
max_bounces = nat.MCV_MAX_BOUNCES


def load_segments(filename):
    """Per-segment h1, h2, w1, w2 from a segment file
    (guide_tapering.py:85-120): one segment per line, "h1 h2 w1 w2"
    separated by single spaces, lines starting with "c" are comments, and
    the last line read is not a segment."""
    h1, h2, w1, w2 = [], [], [], []
    with open(filename) as f:
        for line in f:
            if line.startswith("c"):
                continue
            a, b, c, d = line.split(" ", 3)
            h1.append(a)
            h2.append(b)
            w1.append(c)
            w2.append(d)
    return tuple(np.asarray(v[:-1], dtype=np.float64)
                 for v in (h1, h2, w1, w2))


class Guide(ComponentBase):
    opcode = nat.OP_GUIDE_TAPERING

    # segments per quiet-test block of the kernels (0: segment by segment),
    # used by guides of at least QUIET_MIN_SEGMENTS segments.  Measured
    # (FP32): VERDI's 499-segment mirrors 1.43e8 -> 5.21e8 n/s with blocks
    # of 16 (8: 4.96e8, 32: 4.51e8); a 100-segment guide of 11 cm segments
    # reflects every few segments and ran 8% slower with them.
    QUIET_BLOCK = 16
    QUIET_MIN_SEGMENTS = 256

    def __init__(self, name, option="", l=1.0, mx=2, my=2, R0=0.99,
                 Qcx=0.021, Qcy=0.021, alphax=6.07, alphay=6.07, W=0.003,
                 segments=None, **kwargs):
        """Guide centred on the z axis with its entrance at z=0, of total
        length l (m), cut into equal segments.  option="file={name}" names
        the segment file (as in the reference); `segments` = (h1, h2, w1,
        w2) arrays give them directly.  mx: m of the side mirrors, my: of
        the top and bottom ones (0 absorbs nothing but ends the segment's
        bounces, a negative value scales with the segment's opening)."""
        self.name = name
        self.filename = None
        if option.startswith("file="):
            self.filename = option[len("file="):]
        if segments is None:
            if not self.filename:
                raise RuntimeError("Expected segment file passed to guide")
            segments = load_segments(self.filename)
        h1, h2, w1, w2 = (np.asarray(v, dtype=np.float64) for v in segments)
        self.h1, self.h2, self.w1, self.w2 = h1, h2, w1, w2
        self.nseg = len(h1)
        if self.nseg < 1:
            raise RuntimeError("a tapered guide needs at least one segment")
        self.l_seg = float(l) / self.nseg
        # the data block of prep_inputs_kernel (guide_tapering.py:122-138)
        data = np.zeros((10, self.nseg))
        data[0], data[1], data[2], data[3] = w1, w2, h1, h2
        data[4] = 0.5 * (w2 - w1)           # ww
        data[5] = 0.5 * (h2 - h1)           # hh
        data[6] = 0.5 * w1                  # whalf
        data[7] = 0.5 * h1                  # hhalf
        data[8] = self.l_seg * (0.5 * w1)   # lwhalf
        data[9] = self.l_seg * (0.5 * h1)   # lhhalf
        self.data = data
        scalars = (self.l_seg, R0, Qcx, Qcy, alphax, alphay, mx, my, W)
        self.propagate_params = (self.nseg,
                                 tuple(float(v) for v in scalars), data)

    def quiet_block(self):
        """Segments per quiet-test block for this guide (0: none)."""
        if self.QUIET_BLOCK <= 0 or self.nseg < self.QUIET_MIN_SEGMENTS:
            return 0
        return int(self.QUIET_BLOCK)

    def quiet_blocks(self):
        """Each block of quiet_block() segments' narrowest opening: rows
        min(w1, w2) and min(h1, h2) over the block (the kernels' quiet
        block test)."""
        B = self.quiet_block()
        if B <= 0:
            return np.empty((2, 0))
        nblk = -(-self.nseg // B)
        rows = np.empty((2, nblk))
        for b in range(nblk):
            s = slice(b * B, min((b + 1) * B, self.nseg))
            rows[0, b] = min(self.w1[s].min(), self.w2[s].min())
            rows[1, b] = min(self.h1[s].min(), self.h2[s].min())
        return rows

    def pack(self, c, binder):
        nseg, scalars, data = self.propagate_params
        c.opcode = self.opcode
        c.ip[0] = int(nseg)
        c.ip[1] = self.quiet_block()
        for k, v in enumerate(scalars):
            set_param(c, k, v)
        flat = np.ascontiguousarray(np.concatenate(
            [data.reshape(-1), self.quiet_blocks().reshape(-1)]))
        c.table = binder.table(self, "segments", flat, np.float64)
        c.ftable = binder.table(self, "segments_f32", flat, np.float32)
        c.table_len = flat.size
