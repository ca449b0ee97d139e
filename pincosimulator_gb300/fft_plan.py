"""Register-resident FFT plans for the square-lattice step kernel.

A trajectory of N = 2^n sites (row-major nx x ny, nx = 2^bx rows, ny = 2^by
columns; a chain is bx = 0) is spread over TPT = N / E threads, E = 2^e
elements per thread. The forward transform is a decimation-in-frequency FFT
made of radix-4 (and one trailing radix-2 per odd-sized dimension) stages on
the index bits of each dimension, top bit first; the 2-D transform is the
tensor product of the row and column transforms, as FFTW's 2-D plan computes
(TWMCBaseSolver.cpp:52-60 of the reference). Stages are packed into passes:
in a pass the thread holds the E elements whose positions differ only in the
pass's e "register bits", all stages of the pass run in registers, and
between passes the elements are exchanged through shared memory.

DIF stages leave the spectrum in bit-reversed order within each dimension,
so the k-space multiply reads its table at bit-reversed positions and the
inverse transform (the adjoint stages in reverse order) returns to natural
order without any permutation pass.

`make_plan` is used by build_ext.py to emit the constexpr tables of
csrc/fft_plans.inc, and by the CPU tests, which execute the plan in numpy
against numpy.fft and count shared-memory bank conflicts of every exchange.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np


@dataclass
class Stage:
    dim: int  # 0 = columns (low bits), 1 = rows (high bits)
    t: int  # lowest local bit of the stage
    rb: int  # 2 = radix-4 stage on local bits (t, t+1); 1 = radix-2 on bit t


@dataclass
class Pass:
    reg: list  # global bit of register-slot bit j
    thr: list  # global bit of thread-index bit i
    stages: list = field(default_factory=list)


@dataclass
class Plan:
    nbits: int
    bx: int
    by: int
    e: int
    lo: tuple
    m: tuple
    passes: list

    @property
    def E(self) -> int:
        return 1 << self.e

    @property
    def tpt(self) -> int:
        return 1 << (self.nbits - self.e)


def _stages_for_dim(dim: int, m: int) -> list:
    out = []
    t = m
    while t >= 2:
        out.append(Stage(dim, t - 2, 2))
        t -= 2
    if t == 1:
        out.append(Stage(dim, 0, 1))
    return out


def make_plan(bx: int, by: int, e: int) -> Plan:
    """Plan for an (2^bx x 2^by) lattice with 2^e elements per thread."""
    n = bx + by
    e = min(e, n)
    lo = (0, by)
    m = (by, bx)
    stages = []
    if bx > 0:
        stages += _stages_for_dim(1, bx)
    stages += _stages_for_dim(0, by)
    # Greedy packing of stages into passes of at most e active bits.
    groups = []
    cur, used = [], 0
    for st in stages:
        if used + st.rb > e:
            groups.append(cur)
            cur, used = [], 0
        cur.append(st)
        used += st.rb
    if cur:
        groups.append(cur)
    passes = []
    for gi, g in enumerate(groups):
        active = []
        for st in g:
            active += [lo[st.dim] + st.t + k for k in range(st.rb)]
        active = sorted(active)
        rest = [b for b in range(n) if b not in active]
        # Idle register bits: the highest free bits (keeps the low bits, which
        # index consecutive sites, on threads for coalesced global access).
        idle = sorted(rest, reverse=True)[: e - len(active)]
        reg = sorted(active + idle)
        thr = [b for b in range(n) if b not in reg]
        passes.append(Pass(reg=reg, thr=thr, stages=g))
    return Plan(nbits=n, bx=bx, by=by, e=e, lo=lo, m=m, passes=passes)


# ---------------------------------------------------------------------------
# numpy execution of a plan (exactly the stage arithmetic of the kernel)
# ---------------------------------------------------------------------------
def _stage_apply(x: np.ndarray, plan: Plan, st: Stage, inverse: bool) -> np.ndarray:
    n = plan.nbits
    lo, M = plan.lo[st.dim], 1 << plan.m[st.dim]
    N = 1 << n
    pos = np.arange(N)
    local = (pos >> lo) & (M - 1)
    low = local & ((1 << st.t) - 1)
    y = x.copy()
    if st.rb == 2:
        L = 1 << st.t
        g0 = lo + st.t
        base = pos[((pos >> g0) & 3) == 0]
        lw = low[base]
        w1 = np.exp(-2j * np.pi * lw / (4 * L))
        w2, w3 = w1 ** 2, w1 ** 3
        i0, i1, i2, i3 = base, base + (1 << g0), base + (2 << g0), base + (3 << g0)
        if not inverse:
            x0, x1, x2, x3 = x[i0], x[i1], x[i2], x[i3]
            A, B, C, D = x0 + x2, x1 + x3, x0 - x2, x1 - x3
            y[i0] = A + B
            y[i1] = (A - B) * w2
            y[i2] = (C - 1j * D) * w1
            y[i3] = (C + 1j * D) * w3
        else:
            y0, y1, y2, y3 = x[i0], x[i1], x[i2], x[i3]
            u = np.conj(w2) * y1
            A, B = y0 + u, y0 - u
            p, q = np.conj(w1) * y2, np.conj(w3) * y3
            C, D = p + q, 1j * (p - q)
            y[i0], y[i2], y[i1], y[i3] = A + C, A - C, B + D, B - D
    else:
        L = 1 << st.t
        g0 = lo + st.t
        base = pos[((pos >> g0) & 1) == 0]
        w = np.exp(-2j * np.pi * low[base] / (2 * L))
        i0, i1 = base, base + (1 << g0)
        if not inverse:
            x0, x1 = x[i0], x[i1]
            y[i0], y[i1] = x0 + x1, (x0 - x1) * w
        else:
            u = np.conj(w) * x[i1]
            y[i0], y[i1] = x[i0] + u, x[i0] - u
    return y


def run_forward(plan: Plan, x: np.ndarray) -> np.ndarray:
    y = np.asarray(x, dtype=np.complex128).copy()
    for ps in plan.passes:
        for st in ps.stages:
            y = _stage_apply(y, plan, st, inverse=False)
    return y


def run_inverse(plan: Plan, y: np.ndarray) -> np.ndarray:
    x = np.asarray(y, dtype=np.complex128).copy()
    for ps in reversed(plan.passes):
        for st in reversed(ps.stages):
            x = _stage_apply(x, plan, st, inverse=True)
    return x


def bitrev(v: int, nb: int) -> int:
    r = 0
    for i in range(nb):
        r |= ((v >> i) & 1) << (nb - 1 - i)
    return r


def freq_of_position(plan: Plan):
    """(kx, ky) held at each position after the forward plan (bit reversal per dim)."""
    N = 1 << plan.nbits
    ky = np.array([bitrev(p & ((1 << plan.by) - 1), plan.by) for p in range(N)])
    kx = np.array([bitrev(p >> plan.by, plan.bx) if plan.bx else 0 for p in range(N)])
    return kx, ky


# ---------------------------------------------------------------------------
# shared-memory exchange model
# ---------------------------------------------------------------------------
def swizzle(P: int, nflat_bits: int) -> int:
    """Physical element slot of CTA-flat element P (XOR of bits 4..7 into 0..3)."""
    if nflat_bits < 8:
        return P
    return P ^ ((P >> 4) & 15)


def deposit(v: int, bits: list) -> int:
    r = 0
    for i, b in enumerate(bits):
        r |= ((v >> i) & 1) << b
    return r


def exchange_wavefronts(plan: Plan, k: int, traj_per_cta: int, elem_bytes: int, write: bool) -> float:
    """Average shared-memory wavefronts per warp access of pass k's layout."""
    ps = plan.passes[k]
    n = plan.nbits
    tpt = plan.tpt
    flat_bits = n + max(0, (traj_per_cta - 1).bit_length())
    waves = []
    for w0 in range(0, min(32 * 4, tpt * traj_per_cta), 32):
        for s in range(plan.E):
            banks = {}
            for lane in range(32):
                gt = w0 + lane
                if gt >= tpt * traj_per_cta:
                    continue
                traj, t = divmod(gt, tpt)
                p = deposit(t, ps.thr) | deposit(s, ps.reg)
                phys = swizzle((traj << n) | p, flat_bits)
                byte = phys * elem_bytes
                for wd in range(elem_bytes // 4):
                    bank = (byte // 4 + wd) % 32
                    banks.setdefault(bank, set()).add(byte // 4 + wd)
            worst = max(len(v) for v in banks.values())
            # a 64-bit (128-bit) access needs at least 2 (4) wavefronts per warp
            waves.append(max(worst, elem_bytes // 4))
    return float(np.mean(waves))


SUPPORTED_SHAPES = [
    # (bx, by): 1-D chains N = 32 .. 4096 and 2-D squares L = 16 .. 64
    (0, 5), (0, 6), (0, 7), (0, 8), (0, 9), (0, 10), (0, 11), (0, 12),
    (4, 4), (5, 5), (6, 6),
]


def emit_header(e: int = 4) -> str:
    """C++ source with one constexpr plan per supported shape."""
    lines = ["// Generated by pincosimulator_gb300/fft_plan.py -- do not edit.", "#pragma once", "namespace twmc {"]
    for (bx, by) in SUPPORTED_SHAPES:
        p = make_plan(bx, by, e)
        name = f"Plan_{bx}_{by}"
        lines.append(f"struct {name} {{")
        lines.append(f"  static constexpr int nbits = {p.nbits}, bx = {p.bx}, by = {p.by}, e = {p.e};")
        lines.append(f"  static constexpr int npass = {len(p.passes)};")
        lines.append(f"  static constexpr int lo[2] = {{{p.lo[0]}, {p.lo[1]}}};")
        lines.append(f"  static constexpr int m[2] = {{{p.m[0]}, {p.m[1]}}};")
        regs = ", ".join("{" + ", ".join(str(b) for b in ps.reg) + "}" for ps in p.passes)
        nthr = p.nbits - p.e
        thrs = ", ".join("{" + ", ".join(str(b) for b in (ps.thr if ps.thr else [0])) + "}" for ps in p.passes)
        lines.append(f"  static constexpr int reg[{len(p.passes)}][{p.e}] = {{{regs}}};")
        lines.append(f"  static constexpr int nthr = {nthr};")
        lines.append(f"  static constexpr int thr[{len(p.passes)}][{max(nthr, 1)}] = {{{thrs}}};")
        nst = ", ".join(str(len(ps.stages)) for ps in p.passes)
        lines.append(f"  static constexpr int nst[{len(p.passes)}] = {{{nst}}};")
        st = ", ".join(
            "{" + ", ".join(f"{{{s.dim}, {s.t}, {s.rb}}}" for s in (ps.stages + [Stage(0, 0, 0)] * (4 - len(ps.stages)))) + "}"
            for ps in p.passes
        )
        lines.append(f"  static constexpr int st[{len(p.passes)}][4][3] = {{{st}}};")
        lines.append("};")
    lines.append("}  // namespace twmc")
    return "\n".join(lines) + "\n"
