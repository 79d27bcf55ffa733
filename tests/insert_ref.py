"""NumPy restatement of the device placement generator (test infrastructure): the
Philox4x32-10 stream and the insertion.F90 placement steps, placement by placement."""
import math

import numpy as np

M0, M1, W0, W1 = 0xD2511F53, 0xCD9E8D57, 0x9E3779B9, 0xBB67AE85
MASK = 0xFFFFFFFF


def philox4x32_10(ctr, key):
    c0, c1, c2, c3 = ctr
    k0, k1 = key
    for _ in range(10):
        p0, p1 = M0 * c0, M1 * c2
        c0, c1, c2, c3 = ((p1 >> 32) ^ c1 ^ k0) & MASK, p1 & MASK, ((p0 >> 32) ^ c3 ^ k1) & MASK, p0 & MASK
        k0, k1 = (k0 + W0) & MASK, (k1 + W1) & MASK
    return c0, c1, c2, c3


class Stream:
    def __init__(self, seed, g):
        self.key = (seed & MASK, (seed >> 32) & MASK)
        self.c2, self.c3 = g & MASK, (g >> 32) & MASK
        self.draw = 0
        self.buf = []

    def u32(self):
        if not self.buf:
            self.buf = list(philox4x32_10((self.draw, 0, self.c2, self.c3), self.key))
            self.draw += 1
        return self.buf.pop(0)

    def uniform(self):
        a, b = self.u32() >> 5, self.u32() >> 6
        return (a * 67108864.0 + b) * (1.0 / 9007199254740992.0)


def horn_fit(refa, a, w, b):
    """bestfit.F90 fit_a_rotate_b with numpy's LAPACK eigensolver: a (n, 3) fitted onto refa
    (weights w), the transform applied to b (m, 3)."""
    refa, a, b, w = (np.asarray(v, float) for v in (refa, a, b, w))
    cr = (w[:, None] * refa).sum(0) / w.sum()
    ca = (w[:, None] * a).sum(0) / w.sum()
    S = np.einsum("k,ki,kj->ji", w, refa - cr, a - ca)  # S[j, i] = sum w ref_i a_j
    M = np.array([
        [S[0, 0] + S[1, 1] + S[2, 2], S[1, 2] - S[2, 1], S[2, 0] - S[0, 2], S[0, 1] - S[1, 0]],
        [S[1, 2] - S[2, 1], S[0, 0] - S[1, 1] - S[2, 2], S[0, 1] + S[1, 0], S[2, 0] + S[0, 2]],
        [S[2, 0] - S[0, 2], S[0, 1] + S[1, 0], -S[0, 0] + S[1, 1] - S[2, 2], S[1, 2] + S[2, 1]],
        [S[0, 1] - S[1, 0], S[2, 0] + S[0, 2], S[1, 2] + S[2, 1], -S[0, 0] - S[1, 1] + S[2, 2]]])
    q = np.linalg.eigh(M)[1][:, -1]
    v = b - ca
    u = q[1:]
    t = 2.0 * np.cross(u, v)
    return v + q[0] * t + np.cross(u, t) + cr


def place(bf, mass, cell, p, insposition=0, insorient=0, insorigin=0, lwreg=0.0, upreg=0.0, seed=1, offset=0,
          agg=None, start=None, refbest=None, refw=None, w0=1.0):
    """Placement p.  insorigin 2: agg is the aggregate centre; insorigin 3: start is bfcoord
    fitted onto refbest, the reference solute in the frame, and a draw whose RMSD from it
    (weights refw) lies outside [lwreg, upreg] is drawn again.  w0: the structure's weight
    (a flexible solute's)."""
    g = offset + p
    rng = Stream(seed, g)
    w = w0
    for draw in range(1 << 16):
        x, w = _draw(rng, g + draw, bf if insorigin != 3 else start, mass, cell, insposition, insorient, insorigin,
                     lwreg, upreg, agg, w)
        if insorigin != 3:
            break
        rmsd = math.sqrt(float((refw * ((x - refbest) ** 2).sum(1)).sum() / refw.sum()))
        if not (lwreg > rmsd or rmsd > upreg):
            break
    return x, w


def _draw(rng, parity, x0, mass, cell, insposition, insorient, insorigin, lwreg, upreg, agg, w):
    x = np.array(x0, dtype=float)
    com = lambda y: (mass[:, None] * y).sum(0) / mass.sum()
    if insorigin == 0:
        x = x - com(x)
    elif insorigin == 2:
        x = x - com(x) + agg
    shift = np.zeros(3)
    if insposition == 0:
        r = np.array([rng.uniform() for _ in range(3)])
        shift = cell @ r - com(x)
    elif insposition == 2:
        t = rng.uniform()
        t = (t * (upreg ** 3 - lwreg ** 3) + lwreg ** 3) ** (1.0 / 3.0)
        for _ in range(256):
            r = np.array([rng.uniform() * 2.0 - 1.0 for _ in range(3)])
            n2 = float(r @ r)
            if 0 < n2 <= 1:
                break
        shift = t * r / math.sqrt(n2)
    elif insposition in (3, 4):
        r = np.array([rng.uniform(), rng.uniform(), 0.0])
        t = rng.uniform() * (upreg - lwreg) + lwreg
        if insposition == 4 and rng.uniform() > 0.5:
            t = -t
        r[2] = t / np.linalg.norm(cell[:, 2])
        shift = cell @ r
    elif insposition == 5:
        c = com(x)
        movmax = upreg + 3.0 * math.sqrt(max(float(((x - c) ** 2).sum(1).max()), 0.0))
        shift = np.array([movmax * (2.0 * rng.uniform() - 1.0) for _ in range(3)])
    elif insposition == 6:
        ls = np.linalg.norm(cell, axis=0) / 2.0 / upreg
        z0 = 8 * ls.prod()
        z1 = math.sqrt(math.pi) ** 3 * math.erf(ls[0]) * math.erf(ls[1]) * math.erf(ls[2])
        if parity % 2 == 0:
            sc = np.array([(2 * rng.uniform() - 1) * ls[i] for i in range(3)])
        else:
            sc = np.zeros(3)
            for i in range(3):
                for _ in range(256):
                    r1, r2 = 1 - rng.uniform(), rng.uniform()
                    r = math.sqrt(-2 * math.log(r1)) * math.cos(2 * math.pi * r2) / math.sqrt(2.0)
                    if abs(r) < ls[i]:
                        break
                sc[i] = r
        w = w / (0.5 / z0 + 0.5 * math.exp(-float(sc @ sc)) / z1)
        shift = cell @ (sc / (ls * 2))
    x = x + shift
    if insorient == 0:
        for _ in range(256):
            q = np.array([rng.uniform() * 2.0 - 1.0 for _ in range(4)])
            n2 = float(q @ q)
            if n2 < 1:
                break
        q = q / math.sqrt(n2)
        c = com(x)
        v = x - c
        u = q[1:]
        t = 2.0 * np.cross(u, v)
        x = v + q[0] * t + np.cross(u, t) + c
    return x, w


def rmsd_bestfit(ref, x, w):
    """bestfit.F90 rmsd_bestfit: x fitted onto ref (weights w), then rmsd_nofit."""
    ref, x, w = (np.asarray(v, float) for v in (ref, x, w))
    fitted = horn_fit(ref, x, w, x)
    return math.sqrt(float((w * ((fitted - ref) ** 2).sum(1)).sum() / w.sum()))


def library_accepted(conf, insstructure=0, lwstr=0.0, upstr=0.0, refslt=None, refw=None):
    """getsolute's structure test (insertion.F90:457-470) for every structure of the library:
    the accepted ones, in file order."""
    if insstructure == 0:
        return list(range(len(conf)))
    return [f for f, x in enumerate(conf) if lwstr <= rmsd_bestfit(refslt, x, refw) <= upstr]


def library_pick(g, nconf, acc, nwt):
    """The g-th accepted read of the wrapped structure file: (structure, weight line) -- the
    closed form the device uses."""
    na = len(acc)
    r = (g // na) * nconf + acc[g % na]
    return acc[g % na], (r % nwt if nwt else None)


def library_reads(n, nconf, accepted, nwt):
    """getsolute's loop itself (insertion.F90:432-472), read by read: the structure file and the
    weight file both wrap around, a weight is read with every structure (a rejected one too),
    and a call returns at the first accepted structure.  The first n calls' (structure,
    weight line)."""
    out, r = [], 0
    for _ in range(n):
        while True:
            f, wl = r % nconf, (r % nwt if nwt else None)
            r += 1
            if accepted[f]:
                out.append((f, wl))
                break
    return out
