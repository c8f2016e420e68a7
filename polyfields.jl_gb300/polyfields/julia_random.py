"""Julia's seeded normal stream, so that `fieldinit(sys, seed=s)` writes the fields that the
reference's `fieldinit!(sys; seed = s)` writes (src/fileio.jl:14-23: `Random.seed!(seed)`,
then `omega .= scale * randn(sys.dims)` for each `(mid, omega)` in the `Dict` `sys.fields`).

The reference ran on Julia 1.5/1.6, whose default RNG is `MersenneTwister`.  That is the dSFMT-19937
generator (M. Saito and M. Matsumoto, 2008; MEXP 19937 parameters below), seeded with the
integer's 32-bit words.  It keeps a cache of 1002 doubles in [1, 2), refilled by one block
generation and popped from the front.  Arrays of 384 or more elements are filled by one block
generation straight from the state, with the last few values taken from the cache.
`randn` is the 256-layer ziggurat of Marsaglia and Tsang (2000) on 52 mantissa bits; its
tables are in ziggurat_tables.npz (make_ziggurat_tables.py).  For arrays of 13 or more
elements, `randn!` first draws the whole block, then converts it in order; rejection draws
follow the block.  `Dict{Int}` iterates its slots in order (16, growing to max(16, nextpow2(4 count))
once more than 2/3 are taken); a key's slot is its hash (Thomas Wang's 64-bit mix of
3|x| + bits(Float64(x))) modulo the table size, with linear probing.

The block generation is vectorised: the dSFMT lung obeys lung' = R(lung) ^ c with R an
involution (swap the two 64-bit halves and rotate each by 32 bits), so the lungs of a run of
words are a prefix XOR.  The words of a block depend on the words POS1 - N = -74 places back,
so blocks are generated 74 words at a time.

Streams of arrays up to 383 elements are pinned to the reference's own test goldens through
the oracle's restatement of the same runtime.  Longer arrays follow the fill path just
described, which no golden covers.
"""
from __future__ import annotations

import math
import os
import struct
from typing import Dict, List, Optional, Sequence

import numpy as np

_M32 = (1 << 32) - 1
_N = 191                        # 128-bit state words (+ the lung)
_POS1, _SL1, _SR = 117, 19, 12
_LAG = _N - _POS1               # 74: a block's words depend on words this far back
_MSK = (np.uint64(0x000FFAFFFFFFFB3F), np.uint64(0x000FFDFFFC90FFFD))
_FIX = (0x90014964B32F4329, 0x3B8D12AC548A7C7A)
_PCV = (0x3D84E1AC0DC82880, 0x0000000000000001)
_MANT = 0x000FFFFFFFFFFFFF
_ONE = 0x3FF0000000000000
_CACHE = 1002
_R = 3.6541528853610088
_INV_R = 1.0 / _R

_U32 = np.uint64(32)
_USL1 = np.uint64(_SL1)
_USR = np.uint64(_SR)

_tables = None


def _zig():
    global _tables
    if _tables is None:
        d = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "ziggurat_tables.npz"))
        _tables = (d["k"].astype(np.uint64), d["w"].astype(np.float64), d["f"].astype(np.float64))
    return _tables


def _rot32(x):
    return (x >> _U32) | (x << _U32)


def _init_by_array(key: Sequence[int]):
    """dSFMT initialisation by an array of 32-bit words; returns the state as two uint64 arrays
    (low and high halves of the N + 1 words), masked to [1, 2) and period-certified."""
    n = (_N + 1) * 4
    lag = 11
    mid = (n - lag) // 2
    w = [0x8B8B8B8B] * n

    def f1(x):
        return ((x ^ (x >> 27)) * 1664525) & _M32

    def f2(x):
        return ((x ^ (x >> 27)) * 1566083941) & _M32

    r = f1(w[0] ^ w[mid % n] ^ w[(n - 1) % n])
    w[mid % n] = (w[mid % n] + r) & _M32
    r = (r + len(key)) & _M32
    w[(mid + lag) % n] = (w[(mid + lag) % n] + r) & _M32
    w[0] = r
    i = 1
    for j in range(max(len(key) + 1, n) - 1):
        r = f1(w[i] ^ w[(i + mid) % n] ^ w[(i + n - 1) % n])
        w[(i + mid) % n] = (w[(i + mid) % n] + r) & _M32
        r = (r + (key[j] if j < len(key) else 0) + i) & _M32
        w[(i + mid + lag) % n] = (w[(i + mid + lag) % n] + r) & _M32
        w[i] = r
        i = (i + 1) % n
    for _ in range(n):
        r = f2((w[i] + w[(i + mid) % n] + w[(i + n - 1) % n]) & _M32)
        w[(i + mid) % n] ^= r
        r = (r - i) & _M32
        w[(i + mid + lag) % n] ^= r
        w[i] = r
        i = (i + 1) % n
    u = np.array(w, dtype=np.uint64)
    u64 = u[0::2] | (u[1::2] << _U32)            # N + 1 words x 2 halves, interleaved
    lo, hi = u64[0::2].copy(), u64[1::2].copy()
    lo[:_N] = (lo[:_N] & np.uint64(_MANT)) | np.uint64(_ONE)
    hi[:_N] = (hi[:_N] & np.uint64(_MANT)) | np.uint64(_ONE)
    inner = ((int(lo[_N]) ^ _FIX[0]) & _PCV[0]) ^ ((int(hi[_N]) ^ _FIX[1]) & _PCV[1])
    s = 32
    while s:
        inner ^= inner >> s
        s >>= 1
    if not inner & 1:
        hi[_N] ^= np.uint64(1)
    return lo, hi


class MersenneTwister:
    """Julia's `MersenneTwister(seed)` (non-negative integer seed): raw draws are the IEEE bits of
    doubles in [1, 2)."""

    def __init__(self, seed: int):
        if seed < 0:
            raise ValueError("seed must be non-negative")
        key = []
        while True:
            key.append(seed & _M32)
            seed >>= 32
            if not seed:
                break
        self._lo, self._hi = _init_by_array(key)
        self._cache = np.empty(0, dtype=np.uint64)
        self._next = _CACHE

    def _block(self, m: int) -> np.ndarray:
        """m >= N words of one block generation, as 2 m raw doubles (low, high, low, ...)."""
        slo, shi = self._lo, self._hi
        olo = np.empty(m, dtype=np.uint64)
        ohi = np.empty(m, dtype=np.uint64)
        l0, l1 = slo[_N], shi[_N]
        j0 = 0
        while j0 < m:
            j1 = min(m, j0 + _LAG)
            # a: the word being replaced (state word j, or block word j - N)
            if j1 <= _N:
                alo, ahi = slo[j0:j1], shi[j0:j1]
            elif j0 >= _N:
                alo, ahi = olo[j0 - _N:j1 - _N], ohi[j0 - _N:j1 - _N]
            else:
                alo = np.concatenate([slo[j0:_N], olo[0:j1 - _N]])
                ahi = np.concatenate([shi[j0:_N], ohi[0:j1 - _N]])
            # b: the word POS1 ahead (state word j + POS1 < N, else block word j - LAG)
            if j0 == 0:
                blo, bhi = slo[_POS1:_POS1 + j1], shi[_POS1:_POS1 + j1]
            else:
                blo, bhi = olo[j0 - _LAG:j1 - _LAG], ohi[j0 - _LAG:j1 - _LAG]
            clo = (alo << _USL1) ^ blo
            chi = (ahi << _USL1) ^ bhi
            # g_t = R^t(c_t) (R swaps the halves and rotates each by 32), prefix XOR
            odd = (np.arange(j1 - j0) & 1).astype(bool)
            glo = np.where(odd, _rot32(chi), clo)
            ghi = np.where(odd, _rot32(clo), chi)
            glo = np.bitwise_xor.accumulate(glo)
            ghi = np.bitwise_xor.accumulate(ghi)
            # lung after word t: R^t(R(L) ^ G_t)
            hlo = glo ^ _rot32(l1)
            hhi = ghi ^ _rot32(l0)
            ylo = np.where(odd, _rot32(hhi), hlo)
            yhi = np.where(odd, _rot32(hlo), hhi)
            olo[j0:j1] = (ylo >> _USR) ^ (ylo & _MSK[0]) ^ alo
            ohi[j0:j1] = (yhi >> _USR) ^ (yhi & _MSK[1]) ^ ahi
            l0, l1 = ylo[-1], yhi[-1]
            j0 = j1
        self._lo = np.concatenate([olo[m - _N:], [l0]])
        self._hi = np.concatenate([ohi[m - _N:], [l1]])
        out = np.empty(2 * m, dtype=np.uint64)
        out[0::2] = olo
        out[1::2] = ohi
        return out

    def pops(self, n: int) -> np.ndarray:
        """n raw draws from the cache (refilled by a 501-word block when empty)."""
        parts = []
        while n > 0:
            if self._next >= _CACHE:
                self._cache = self._block(_CACHE // 2)
                self._next = 0
            take = min(n, _CACHE - self._next)
            parts.append(self._cache[self._next:self._next + take])
            self._next += take
            n -= take
        return np.concatenate(parts) if parts else np.empty(0, dtype=np.uint64)

    def rand(self) -> float:
        """`rand(rng)`: one double in [0, 1)."""
        return struct.unpack("<d", struct.pack("<Q", int(self.pops(1)[0])))[0] - 1.0

    def raw_array(self, n: int) -> np.ndarray:
        """`rand!(rng, A, CloseOpen12())` for n doubles, as raw bits."""
        n2 = (n - 2) // 2 * 2
        if n2 < 2 * _N:
            return self.pops(n)
        return np.concatenate([self._block(n2 // 2), self.pops(n - n2)])

    def _convert(self, bits: int) -> float:
        """One ziggurat conversion; rejections draw more from this generator."""
        k, w, f = _zig()
        bits &= _MANT
        mag = bits >> 1
        layer = mag & 0xFF
        x = float(-mag if bits & 1 else mag) * float(w[layer])
        if mag < int(k[layer]):
            return x
        if layer == 0:
            while True:
                xx = -_INV_R * math.log(self.rand())
                yy = -math.log(self.rand())
                if yy + yy > xx * xx:
                    return float(-(_R + xx) if (mag >> 8) & 1 else _R + xx)
        if (float(f[layer - 1]) - float(f[layer])) * self.rand() + float(f[layer]) < math.exp(-0.5 * x * x):
            return x
        return self.randn()

    def randn(self) -> float:
        """`randn(rng)`: one standard normal."""
        return self._convert(int(self.pops(1)[0]))

    def randn_array(self, n: int) -> np.ndarray:
        """`randn!(rng, A)` for n doubles in linear (column-major) order."""
        if n < 13:
            return np.array([self.randn() for _ in range(n)], dtype=np.float64)
        k, w, _ = _zig()
        bits = self.raw_array(n) & np.uint64(_MANT)
        mag = bits >> np.uint64(1)
        layer = (mag & np.uint64(0xFF)).astype(np.intp)
        signed = np.where((bits & np.uint64(1)).astype(bool), -mag.astype(np.int64), mag.astype(np.int64))
        out = signed.astype(np.float64) * w[layer]
        for i in np.nonzero(mag >= k[layer])[0]:   # in order: their rejection draws follow the block
            out[i] = self._convert(int(bits[i]))
        return out


def _wang64(a: int) -> int:
    m = (1 << 64) - 1
    a = ((~a & m) + (a << 21)) & m
    a ^= a >> 24
    a = (a + (a << 3) + (a << 8)) & m
    a ^= a >> 14
    a = (a + (a << 2) + (a << 4)) & m
    a ^= a >> 28
    return (a + (a << 31)) & m


def _slot_hash(key: int) -> int:
    fbits = struct.unpack("<Q", struct.pack("<d", float(key)))[0]
    return _wang64((3 * abs(key) + fbits) & ((1 << 64) - 1))


def dict_order(keys: Sequence[int]) -> List[int]:
    """Iteration order of a Julia `Dict{Int}` holding `keys` (inserted in this order): 16
    slots, linear probing, and a rehash into max(16, nextpow2(4 count)) slots (keys reinserted
    in slot order) once more than 2/3 of the slots are taken."""
    table: List[Optional[int]] = [None] * 16

    def place(slots: List[Optional[int]], key: int) -> None:
        m = len(slots) - 1
        i = _slot_hash(key) & m
        while slots[i] is not None:
            i = (i + 1) & m
        slots[i] = key

    count = 0
    for key in keys:
        if key in table:
            continue
        place(table, key)
        count += 1
        if 3 * count > 2 * len(table):
            grown: List[Optional[int]] = [None] * max(16, 1 << (4 * count - 1).bit_length())
            for k in table:
                if k is not None:
                    place(grown, k)
            table = grown
    return [k for k in table if k is not None]


_global: Optional[MersenneTwister] = None


def default_rng(seed: int = -1) -> MersenneTwister:
    """The process-wide generator of fieldinit: `Random.seed!(seed)` for seed >= 0, else the
    current stream (seeded from the OS on first use, as Julia's default RNG is)."""
    global _global
    if seed >= 0:
        _global = MersenneTwister(seed)
    elif _global is None:
        _global = MersenneTwister(int.from_bytes(os.urandom(16), "little"))
    return _global


def fieldinit_fields(mids: Sequence[int], shape, seed: int = -1, scale: float = 0.1) -> Dict[int, np.ndarray]:
    """The fields of `fieldinit!(sys; seed, scale)` for a system whose monomers were added with
    ids `mids` (in that order), on a grid of `shape` (Nz, Ny, Nx)."""
    rng = default_rng(seed)
    n = int(np.prod(shape))
    return {mid: scale * rng.randn_array(n).reshape(shape) for mid in dict_order(list(mids))}
