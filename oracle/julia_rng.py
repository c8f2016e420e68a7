"""Test infrastructure (oracle side): the random fields of the reference's `fieldinit!(sys;
seed, scale)` (src/fileio.jl:14-23), restated so that the reference's own RNG-dependent test
goldens (test/test_system.jl:29-34, test/test_updaters.jl:24-30) can be checked here.

`fieldinit!` runs `Random.seed!(seed)` and then, for each `(mid, omega)` in `sys.fields` (a
`Dict{Int, Array}`, src/system/system.jl:35), `omega .= scale * randn(sys.dims)`.  Three pieces of
the Julia runtime the reference was written against (Julia 1.5/1.6; the default RNG became
Xoshiro in 1.7) decide the values.  That runtime is a third-party dependency absent from the
reference tree, so each piece is restated here from its published algorithm:

1. The default RNG, `MersenneTwister`: the double-precision SIMD-oriented Fast Mersenne
   Twister dSFMT-19937 (M. Saito and M. Matsumoto, "SIMD-oriented Fast Mersenne Twister: a
   128-bit pseudorandom number generator", 2008, and the dSFMT 2.x reference implementation,
   whose MEXP 19937 parameters are the constants below).  Julia seeds it with the integer's
   32-bit words (init by array), keeps a cache of 1002 doubles in [1, 2) that it refills by
   one block generation and pops from the front.
2. `randn`: the 256-layer ziggurat of G. Marsaglia and W. W. Tsang ("The Ziggurat Method for
   Generating Random Variables", J. Stat. Softw. 5(8), 2000) on 52 random mantissa bits: bit 0
   is the sign, bits 1..8 the layer, bits 1..51 the abscissa.  The layer tables use the right
   edge r = 3.6541528853610088 and a layer area v that is computed exactly from r (below,
   in 50-digit arithmetic).  For a `Float64` array of 13 or more elements, `randn!` first
   takes one raw draw per element, then converts them in order.  Any rejection draws a
   conversion needs come after the whole block.  The raw draws come from the cache for
   arrays of up to 383 elements.  Longer arrays are generated straight from the state (see
   `MersenneTwister.raw_array`); that path follows the same runtime but no golden pins it.
3. `Dict` iteration order: slots in ascending order, a key's home slot is
   `hash(key) & (sz - 1)` in a table of 16 slots (grown when over 2/3 full), with linear
   probing; `hash(::Int64)` is
   Thomas Wang's 64-bit integer mix of `3|x| + bits(Float64(x))`.  For monomer ids (1, 2, 3)
   the order is (2, 3, 1); for (1, 2) it is (2, 1).

Checks that pin this restatement (tests/test_julia_seed_goldens.py):
* `rand(MersenneTwister(1234))` and `randn(MersenneTwister(1234))` equal the values that
  Julia's manual prints for them.
* With these fields, the FP64 oracle reproduces all five goldens of test/test_system.jl to
  within 2e-15, and the Euler golden of test/test_updaters.jl to the last digit.  It also
  reproduces that file's commented-out NAG value at 3e-15.  Its Anderson golden matches at
  3e-10, inside the reference test's own `isapprox` tolerance of sqrt(eps) = 1.5e-8.  The
  Anderson step solves a least-squares system on nearly collinear residual histories, which
  amplifies the last-bit differences between this FFT and FFTW.

Nothing in the engine imports this module.  Only the fixture generator
(tests/golden/make_julia_seed_fields.py) and the tests do.
"""
from __future__ import annotations

import math
import struct
from typing import Dict, List, Sequence, Tuple

_M64 = (1 << 64) - 1
_M32 = (1 << 32) - 1

# ----------------------------------------------------------------------------- dSFMT-19937
_NW = 191                     # 128-bit words in the state (plus one "lung" word)
_POS1, _SL1, _SR = 117, 19, 12
_MSK = (0x000FFAFFFFFFFB3F, 0x000FFDFFFC90FFFD)
_FIX = (0x90014964B32F4329, 0x3B8D12AC548A7C7A)
_PCV = (0x3D84E1AC0DC82880, 0x0000000000000001)
_MANT = 0x000FFFFFFFFFFFFF    # 52 mantissa bits
_ONE = 0x3FF0000000000000     # exponent bits of a double in [1, 2)
_CACHE = 1002                 # doubles per refill of Julia's MersenneTwister cache


def _step(a, b, lung):
    """The affine recursion of dSFMT: new word from a (the word being replaced), b (the word
    POS1 ahead) and the lung; returns (word, new lung).  Words are (low, high) 64-bit pairs."""
    l0, l1 = lung
    y0 = ((a[0] << _SL1) & _M64) ^ (l1 >> 32) ^ ((l1 << 32) & _M64) ^ b[0]
    y1 = ((a[1] << _SL1) & _M64) ^ (l0 >> 32) ^ ((l0 << 32) & _M64) ^ b[1]
    return ((y0 >> _SR) ^ (y0 & _MSK[0]) ^ a[0], (y1 >> _SR) ^ (y1 & _MSK[1]) ^ a[1]), (y0, y1)


def _seed_words(key: Sequence[int]) -> List[Tuple[int, int]]:
    """dSFMT's initialisation by an array of 32-bit words, followed by the mask that puts every
    state double in [1, 2) and the period certification of the lung."""
    n = (_NW + 1) * 4                     # 32-bit words, lung included
    lag = 11
    mid = (n - lag) // 2
    w = [0x8B8B8B8B] * n

    def mix1(x):
        return ((x ^ (x >> 27)) * 1664525) & _M32

    def mix2(x):
        return ((x ^ (x >> 27)) * 1566083941) & _M32

    def at(i):
        return i % n

    rounds = max(len(key) + 1, n)
    r = mix1(w[0] ^ w[at(mid)] ^ w[at(n - 1)])
    w[at(mid)] = (w[at(mid)] + r) & _M32
    r = (r + len(key)) & _M32
    w[at(mid + lag)] = (w[at(mid + lag)] + r) & _M32
    w[0] = r
    i = 1
    for j in range(rounds - 1):
        r = mix1(w[i] ^ w[at(i + mid)] ^ w[at(i + n - 1)])
        w[at(i + mid)] = (w[at(i + mid)] + r) & _M32
        r = (r + (key[j] if j < len(key) else 0) + i) & _M32
        w[at(i + mid + lag)] = (w[at(i + mid + lag)] + r) & _M32
        w[i] = r
        i = at(i + 1)
    for _ in range(n):
        r = mix2((w[i] + w[at(i + mid)] + w[at(i + n - 1)]) & _M32)
        w[at(i + mid)] ^= r
        r = (r - i) & _M32
        w[at(i + mid + lag)] ^= r
        w[i] = r
        i = at(i + 1)
    u = [w[2 * k] | (w[2 * k + 1] << 32) for k in range(2 * (_NW + 1))]
    for k in range(2 * _NW):
        u[k] = (u[k] & _MANT) | _ONE
    words = [(u[2 * k], u[2 * k + 1]) for k in range(_NW + 1)]
    t0, t1 = words[_NW][0] ^ _FIX[0], words[_NW][1] ^ _FIX[1]
    parity = (t0 & _PCV[0]) ^ (t1 & _PCV[1])
    s = 32
    while s:
        parity ^= parity >> s
        s >>= 1
    if not parity & 1:
        words[_NW] = (words[_NW][0], words[_NW][1] ^ 1)  # PCV2 has bit 0 set
    return words


class MersenneTwister:
    """Julia's `MersenneTwister(seed)` for a non-negative integer seed, drawing doubles in
    [1, 2) (as raw IEEE bits) from its 1002-entry cache."""

    def __init__(self, seed: int):
        if seed < 0:
            raise ValueError("seed must be non-negative")
        key = []
        while True:
            key.append(seed & _M32)
            seed >>= 32
            if seed == 0:
                break
        self._state = _seed_words(key)
        self._cache: List[int] = []
        self._next = _CACHE

    def _block(self, m: int) -> List[int]:
        """Block generation of m >= _NW words (2 m doubles as raw bits): the first _NW words
        come from the state, later ones from the block itself; the state becomes the block's
        last _NW words."""
        st = self._state
        lung = st[_NW]
        out: List[Tuple[int, int]] = []
        for i in range(m):
            a = st[i] if i < _NW else out[i - _NW]
            k = i + _POS1
            b = st[k] if k < _NW else out[k - _NW]
            word, lung = _step(a, b, lung)
            out.append(word)
        self._state = out[m - _NW:] + [lung]
        return [x for word in out for x in word]

    def _refill(self):
        self._cache = self._block(_CACHE // 2)
        self._next = 0

    def raw_array(self, n: int) -> List[int]:
        """`rand!(rng, A, CloseOpen12())` for a Float64 array of n elements.  Up to n2 =
        2 floor((n - 2) / 2) < 382: n draws from the cache.  Larger: n2 values by one block
        generation straight from the state (the cache is left as it is), then n - n2 from
        the cache.  (The first path is the one the reference's goldens pin; no golden here
        covers the second.)"""
        n2 = (n - 2) // 2 * 2
        if n2 < 2 * _NW:
            return [self.raw() for _ in range(n)]
        return self._block(n2 // 2) + [self.raw() for _ in range(n - n2)]

    def raw(self) -> int:
        """IEEE bits of the next double in [1, 2)."""
        if self._next >= _CACHE:
            self._refill()
        v = self._cache[self._next]
        self._next += 1
        return v

    def rand(self) -> float:
        """`rand(rng)`: a double in [0, 1)."""
        return struct.unpack("<d", struct.pack("<Q", self.raw()))[0] - 1.0


# ----------------------------------------------------------------------------- ziggurat
_R = 3.6541528853610088
_INV_R = 1.0 / _R   # the tail sampler multiplies by 1/r


def _ziggurat_tables():
    """Layer thresholds k (integers on the 51-bit abscissa scale), widths w and heights f of
    the 256-layer normal ziggurat, in 50-digit arithmetic and rounded once."""
    import mpmath as mp
    with mp.workdps(50):
        r = mp.mpf(_R)
        v = r * mp.exp(-r * r / 2) + mp.sqrt(mp.pi / 2) * mp.erfc(r / mp.sqrt(2))
        scale = mp.mpf(2) ** 51
        k = [0] * 256
        w = [0.0] * 256
        f = [0.0] * 256
        x = r
        base = v / mp.exp(-x * x / 2)     # width of the bottom layer including its tail
        k[0] = int(mp.floor(x / base * scale))
        w[0] = float(base / scale)
        w[255] = float(x / scale)
        f[0] = 1.0
        f[255] = float(mp.exp(-x * x / 2))
        for i in range(254, 0, -1):
            inner = mp.sqrt(-2 * mp.log(v / x + mp.exp(-x * x / 2)))
            k[i + 1] = int(mp.floor(inner / x * scale))
            f[i] = float(mp.exp(-inner * inner / 2))
            w[i] = float(inner / scale)
            x = inner
    return k, w, f


_TABLES = None


def _tables():
    global _TABLES
    if _TABLES is None:
        _TABLES = _ziggurat_tables()
    return _TABLES


def _normal_from_bits(rng: MersenneTwister, bits: int) -> float:
    """One ziggurat conversion of 52 raw bits; rejections draw more from rng."""
    k, w, f = _tables()
    bits &= _MANT
    mag = bits >> 1
    layer = mag & 0xFF
    x = (-mag if bits & 1 else mag) * w[layer]
    if mag < k[layer]:
        return x
    if layer == 0:                        # the tail beyond r
        while True:
            xx = -_INV_R * math.log(rng.rand())
            yy = -math.log(rng.rand())
            if yy + yy > xx * xx:
                return -(_R + xx) if (mag >> 8) & 1 else _R + xx
    if (f[layer - 1] - f[layer]) * rng.rand() + f[layer] < math.exp(-0.5 * x * x):
        return x                          # the wedge of this layer
    return randn(rng)


def randn(rng: MersenneTwister) -> float:
    """`randn(rng)` for one Float64."""
    return _normal_from_bits(rng, rng.raw())


def randn_array(rng: MersenneTwister, n: int) -> List[float]:
    """`randn!(rng, A)` for a Float64 array of n elements, in linear (column-major) order."""
    if n < 13:
        return [randn(rng) for _ in range(n)]
    block = rng.raw_array(n)
    return [_normal_from_bits(rng, b) for b in block]


# ----------------------------------------------------------------------------- Dict order
def _wang64(a: int) -> int:
    a = ((~a & _M64) + (a << 21)) & _M64
    a ^= a >> 24
    a = (a + (a << 3) + (a << 8)) & _M64
    a ^= a >> 14
    a = (a + (a << 2) + (a << 4)) & _M64
    a ^= a >> 28
    return (a + (a << 31)) & _M64


def _hash_int(x: int) -> int:
    fbits = struct.unpack("<Q", struct.pack("<d", float(x)))[0]
    return _wang64((3 * abs(x) + fbits) & _M64)


def dict_order(keys: Sequence[int]) -> List[int]:
    """Iteration order of a Julia `Dict{Int, V}` filled with `keys` in this order: 16 slots to
    start, linear probing from the home slot, and once more than 2/3 of the slots are taken a
    rehash into max(16, nextpow2(4 count)) slots that reinserts the keys in slot order.  (The
    reference's systems have a handful of monomers; beyond 10 keys no golden pins this.)"""
    def place(slots, key):
        m = len(slots) - 1
        i = _hash_int(key) & m
        while slots[i] is not None:
            i = (i + 1) & m
        slots[i] = key

    slots: List = [None] * 16
    count = 0
    for key in keys:
        if key in slots:
            continue
        place(slots, key)
        count += 1
        if 3 * count > 2 * len(slots):
            grown: List = [None] * max(16, 1 << (4 * count - 1).bit_length())
            for k in slots:
                if k is not None:
                    place(grown, k)
            slots = grown
    return [s for s in slots if s is not None]


# ----------------------------------------------------------------------------- fieldinit!
def fieldinit_fields(mids: Sequence[int], dims: Sequence[int], seed: int, scale: float = 0.1) -> Dict[int, list]:
    """The fields `fieldinit!(sys; seed, scale)` writes for a system whose monomers were added
    with ids `mids` (in that order) on grid `dims` (Nx, Ny, Nz): per id, scale * randn values in
    column-major order (x fastest), i.e. row-major over (Nz, Ny, Nx)."""
    rng = MersenneTwister(seed)
    n = 1
    for d in dims:
        n *= int(d)
    out = {}
    for mid in dict_order(list(mids)):
        out[mid] = [scale * v for v in randn_array(rng, n)]
    return out
