"""CPU model of the scan kernel's arithmetic (test infrastructure).

Re-derives, in plain Python integers, every table the device uses (sorted inner ring, 32-bit
carry-split keys and buckets, ring-1 residues, word-mask phases, wrap corrections) and walks
positions exactly the way es_scan_kernel does: b2 from rings >= 2, one ring-1 term, the carry
split of the inner ring, the word-mask stage over the first F filters, the residue stage over
the next four, then the exact tail.
It isolates "the decomposition is wrong" from "the CUDA is wrong", like the reference's CPU
emulation of its kernel index scheme (tests/test_enumeration.py).
"""
from __future__ import annotations


class KernelModel:
    def __init__(self, plan, F: int = 4):
        M = plan.M
        self.k, self.M = plan.k, M
        terms = [[(a * b) % M for a in res] for (_, res), b in zip(plan.rings, plan.basis)]
        while len(terms) < 3:
            terms.append([0])
        self.terms = terms
        self.r0, self.r1, self.r2 = len(terms[0]), len(terms[1]), len(terms[2])
        self.radix = [len(t) for t in terms]
        order = sorted(range(self.r0), key=lambda i: terms[0][i])
        self.S0 = [terms[0][i] for i in order]
        self.I0 = order
        bl = M.bit_length()
        self.sh = bl - 32 if bl > 32 else 0
        self.K0 = [v >> self.sh for v in self.S0] + [0xFFFFFFFF]      # sentinel
        kb = (M >> self.sh).bit_length()
        self.bsh = kb - 9 if kb > 9 else 0                  # 512 buckets
        self.BK = [sum(1 for x in self.K0[:-1] if x < (b << self.bsh)) for b in range(513)]
        # the device's 16-byte bucket entry: first slot and the keys of it and the next two
        pad = self.K0 + [0xFFFFFFFF] * 2
        self.BKX = [(n, pad[n], pad[n + 1], pad[n + 2]) for n in self.BK]
        self.K1 = [v >> self.sh for v in terms[1]]       # 32-bit keys of the ring-1 terms
        self.KM = M >> self.sh
        self.exact_fallbacks = 0
        self.q = [plan.info[p][0] for p in plan.rest]
        self.ok = [set(plan.info[p][1]) for p in plan.rest]
        self.corr = [(q - M % q) % q for q in self.q]
        self.F = min(F, len(self.q))
        # filters of the residue stage: the next four that carry 32-bit term residues
        self.FR = max(self.F, min(8, len(self.q), self.F + 4))
        self.W = (self.r0 + 31) // 32

    def wrap_and_split(self, b2: int, d1: int) -> tuple[bool, int]:
        """The kernel's ring-1 wrap and inner carry split from 32-bit keys (no 128-bit math on
        the common path): A = M - b2 once per cycle; t = KA - K1[d1] (+ KM on a wrap) is the key
        of thr = M - b to within +-1; slots keyed outside that band are decided by their keys,
        the rest by exact comparison."""
        M, sh = self.M, self.sh
        A = M - b2
        KA = A >> sh
        k1 = self.K1[d1]
        w1 = k1 > KA
        t = self.KM - (k1 - KA) if w1 else KA - k1
        assert 0 <= t <= 0xFFFFFFFF or k1 == KA
        tl = max(t, 1) - 1
        th = min(t, 0xFFFFFFFE) + 1
        n, ka, kb, kc = self.BKX[tl >> self.bsh]
        s = n + (ka < tl) + (kb < tl)
        ks = kc if kb < tl else (kb if ka < tl else ka)
        assert ks == self.K0[s]
        if k1 == KA or ks <= th:
            self.exact_fallbacks += 1
            w1 = self.terms[1][d1] >= A
            b = b2 + self.terms[1][d1] - (M if w1 else 0)
            thr = M - b
            te = thr >> sh
            s = self.BK[te >> self.bsh]
            sent = self.S0 + [M]
            while self.K0[s] < te:
                s += 1
            while self.K0[s] == te and sent[s] < thr:
                s += 1
        return w1, s

    def b2(self, c: int) -> int:
        rem, acc = c, 0
        for j in range(2, len(self.terms)):
            rem, d = divmod(rem, self.radix[j])
            acc = (acc + self.terms[j][d]) % self.M
        return acc

    def scan(self, t: int, outer) -> tuple[list[int], list[int]]:
        M, r0 = self.M, self.r0
        nf = len(self.q)
        tc = [((t % q) * (M % q)) % q for q in self.q]
        counts = [0] * nf
        surv = []
        for oidx in outer:
            c, d1 = divmod(int(oidx), self.r1)
            b2 = self.b2(c)
            BQ2 = [(b2 % q + tc[f]) % q for f, q in enumerate(self.q[:self.F])]
            BQx = {f: (b2 % self.q[f] + tc[f]) % self.q[f] for f in range(self.F, self.FR)}
            s1 = b2 + self.terms[1][d1]
            w1, sp = self.wrap_and_split(b2, d1)
            assert w1 == (s1 >= M), "ring-1 wrap"
            b = s1 - M if w1 else s1
            assert sp == sum(1 for v in self.S0 if v + b < M), "carry split"
            for wd in range(self.W):
                n_here = min(32, r0 - 32 * wd)
                bits = (1 << n_here) - 1
                cm = sum(1 << i for i in range(n_here) if 32 * wd + i >= sp)
                for f in range(self.F):
                    q = self.q[f]
                    x0 = (BQ2[f] + self.terms[1][d1] % q + (self.corr[f] if w1 else 0)) % q
                    x1 = (x0 + self.corr[f]) % q
                    m0 = sum(1 << i for i in range(n_here) if (x0 + self.S0[32 * wd + i]) % q in self.ok[f])
                    m1 = sum(1 << i for i in range(n_here) if (x1 + self.S0[32 * wd + i]) % q in self.ok[f])
                    bits &= (m0 & ~cm) | (m1 & cm)
                    counts[f] += bin(bits).count("1")
                for i in range(n_here):
                    if not (bits >> i) & 1:
                        continue
                    slot = 32 * wd + i
                    s = (b + self.S0[slot]) % M
                    cw = (cm >> i) & 1
                    ok = True
                    # residue stage (the flush): 32-bit residues of b2, the ring-1 term and the
                    # inner term, with -M mod q per wrap; each sum stays below 3q
                    for f in range(self.F, self.FR):
                        q, corr = self.q[f], self.corr[f]
                        x = BQx[f] + self.terms[1][d1] % q + (corr if w1 else 0)
                        assert x < 3 * q
                        x %= q
                        x = x + self.S0[slot] % q + (corr if cw else 0)
                        assert x < 3 * q
                        x %= q
                        assert x == (s % q + tc[f]) % q, "residue stage"
                        if x not in self.ok[f]:
                            ok = False
                            break
                        counts[f] += 1
                    if not ok:
                        continue
                    for f in range(self.FR, nf):
                        if (s % self.q[f] + tc[f]) % self.q[f] not in self.ok[f]:
                            ok = False
                            break
                        counts[f] += 1
                    if ok:
                        surv.append(int(oidx) * r0 + self.I0[slot])
        return sorted(surv), counts


def units_of(c_begin: int, c_end: int, r2: int, strip: int) -> int:
    """Warp-units of the ring-1 cycles [c_begin, c_end) (csrc/es_abi.cu units_of)."""
    if c_end <= c_begin:
        return 0
    if r2 <= 1:
        return -(-(c_end - c_begin) // (32 * strip))
    rows = -(-c_end // r2) - c_begin // r2
    return -(-rows // 32) * -(-r2 // strip)


def unit_cycles(u: int, lane: int, c_begin: int, c_end: int, r2: int, strip: int) -> list[int]:
    """The cycles lane `lane` of warp-unit `u` scans, in step order (scan_unit in
    csrc/es_scan_kernel.cuh): with a ring 2, rows row0 + 32 (u // J) + lane over the balanced
    digit window j = u mod J of J = ceil(r2 / strip); without one, `strip` consecutive cycles
    per lane."""
    if r2 > 1:
        J = -(-r2 // strip)
        rb, j = divmod(u, J)
        wlo, whi = j * r2 // J, (j + 1) * r2 // J
        e_lo = (c_begin // r2 + 32 * rb) * r2 + wlo + lane * r2
        return [e for e in range(e_lo, e_lo + (whi - wlo)) if c_begin <= e < c_end]
    e_lo = c_begin + (32 * u + lane) * strip
    return [e for e in range(e_lo, e_lo + strip) if e < c_end]


def pair_entry(d1: int, split_lo: int, wrap_lo: bool, split_hi: int, wrap_hi: bool, lane: int) -> tuple[int, int]:
    """Fields z, w of a queue entry holding the words of ring-1 digits d1 (even) and d1 + 1 of a
    one-word inner ring (push in csrc/es_scan_kernel.cuh)."""
    return d1 | split_lo << 16 | split_hi << 24, lane | int(wrap_lo) << 5 | int(wrap_hi) << 6


def pair_candidate(z: int, w: int, i: int) -> tuple[int, int, int, bool, int]:
    """(d1, slot, split, wrap, lane) of candidate bit i in [0, 64) of a paired entry (flush)."""
    hw = i >> 5
    split = (z >> 24) if hw else (z >> 16) & 0xFF
    return (z & 0xFFFF) + hw, i & 31, split, bool((w >> (5 + hw)) & 1), w & 31
