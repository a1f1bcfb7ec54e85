"""The random stream of the reference plugin's start-up scene.

The reference draws its start-up velocities with
``ChaCha8Rng::seed_from_u64(0)`` and ``rng.gen_range(-0.8..0.8)`` for f32
(src/physics/mod.rs:198-212), from the crates rand 0.8.5, rand_core 0.6.4 and
rand_chacha 0.3.1 (Cargo.lock:3681-3705; not vendored).  This module restates
the published algorithms those crates implement:

* ``seed_from_u64`` (rand_core's default): the 32-byte seed is filled with
  successive outputs of a PCG32 step (LCG multiplier 6364136223846793005,
  increment 11634580027462260723, state advanced before each output; output
  xorshift ((s >> 18) ^ s) >> 27 rotated right by s >> 59), each written
  little-endian.
* ChaCha with 8 rounds (Bernstein, "ChaCha, a variant of Salsa20", 2008): the
  16-word state is the four constants "expand 32-byte k", the eight key words
  (the seed, little-endian), a 64-bit block counter in words 12-13 starting at 0
  and a 64-bit stream id in words 14-15 (0).  Each block's output is the 16
  words of (rounds(state) + state), in order; blocks follow the counter.
* ``next_u32`` returns the stream's words in order.
* rand 0.8's single-sample uniform f32 in [low, high): take a u32, keep its
  high 23 bits as the mantissa of a float in [1, 2), subtract 1, then
  ``value * (high - low) + low`` with two f32 roundings (no fused multiply-add);
  a result that rounds up to ``high`` is drawn again (for finite bounds the
  scale stays as it is).

The ChaCha core is checked against the published ChaCha20 zero-key test vector
(tests/test_chacha.py); the seeding and sampling steps follow the crates'
published source and cannot be run here (no Rust toolchain), so the stream is
unpinned against the reference itself.
"""

from __future__ import annotations

import numpy as np

_MASK = 0xFFFFFFFF
_SIGMA = (0x61707865, 0x3320646E, 0x79622D32, 0x6B206574)  # "expand 32-byte k"


def _rotl(x: np.ndarray, r: int) -> np.ndarray:
    return ((x << np.uint32(r)) | (x >> np.uint32(32 - r))).astype(np.uint32)


def chacha_blocks(key_words, counter0: int, count: int, rounds: int = 8, stream: int = 0) -> np.ndarray:
    """`count` consecutive ChaCha blocks (block counters counter0, counter0 + 1, ...)
    as a (count, 16) uint32 array."""
    ctr = np.arange(counter0, counter0 + count, dtype=np.uint64)
    init = np.zeros((16, count), np.uint32)
    for i, c in enumerate(_SIGMA):
        init[i] = c
    for i in range(8):
        init[4 + i] = np.uint32(key_words[i])
    init[12] = (ctr & np.uint64(_MASK)).astype(np.uint32)
    init[13] = (ctr >> np.uint64(32)).astype(np.uint32)
    init[14] = np.uint32(stream & _MASK)
    init[15] = np.uint32((stream >> 32) & _MASK)
    x = [init[i].copy() for i in range(16)]

    def qr(a, b, c, d):
        x[a] = x[a] + x[b]; x[d] = _rotl(x[d] ^ x[a], 16)
        x[c] = x[c] + x[d]; x[b] = _rotl(x[b] ^ x[c], 12)
        x[a] = x[a] + x[b]; x[d] = _rotl(x[d] ^ x[a], 8)
        x[c] = x[c] + x[d]; x[b] = _rotl(x[b] ^ x[c], 7)

    with np.errstate(over="ignore"):
        for _ in range(rounds // 2):
            qr(0, 4, 8, 12); qr(1, 5, 9, 13); qr(2, 6, 10, 14); qr(3, 7, 11, 15)
            qr(0, 5, 10, 15); qr(1, 6, 11, 12); qr(2, 7, 8, 13); qr(3, 4, 9, 14)
        out = np.stack([x[i] + init[i] for i in range(16)], axis=1)
    return out.astype(np.uint32)


def pcg32_seed_bytes(state: int, nbytes: int = 32) -> bytes:
    """rand_core's seed_from_u64 fill: PCG32 outputs, little-endian, state advanced first."""
    mul, inc = 6364136223846793005, 11634580027462260723
    out = bytearray()
    s = state & 0xFFFFFFFFFFFFFFFF
    while len(out) < nbytes:
        s = (s * mul + inc) & 0xFFFFFFFFFFFFFFFF
        xorshifted = (((s >> 18) ^ s) >> 27) & _MASK
        rot = s >> 59
        x = ((xorshifted >> rot) | (xorshifted << ((32 - rot) & 31))) & _MASK
        out += x.to_bytes(4, "little")
    return bytes(out[:nbytes])


class ChaCha8Rng:
    """ChaCha8Rng::seed_from_u64(seed): next_u32 over the block stream."""

    def __init__(self, seed: int):
        key = pcg32_seed_bytes(seed, 32)
        self.key = [int.from_bytes(key[4 * i:4 * i + 4], "little") for i in range(8)]
        self._buf = np.zeros(0, np.uint32)
        self._pos = 0
        self._next_block = 0

    def words(self, count: int) -> np.ndarray:
        """The next `count` u32 outputs."""
        while self._buf.size - self._pos < count:
            need = count - (self._buf.size - self._pos)
            blocks = max(4, (need + 15) // 16)
            fresh = chacha_blocks(self.key, self._next_block, blocks).reshape(-1)
            self._next_block += blocks
            self._buf = np.concatenate([self._buf[self._pos:], fresh])
            self._pos = 0
        out = self._buf[self._pos:self._pos + count].copy()
        self._pos += count
        return out

    def next_u32(self) -> int:
        return int(self.words(1)[0])


def uniform_f32(rng: ChaCha8Rng, low: float, high: float) -> np.float32:
    """rand 0.8 ``gen_range(low..high)`` for f32 (UniformFloat single sample)."""
    lo, hi = np.float32(low), np.float32(high)
    scale = np.float32(hi - lo)
    if not (np.isfinite(lo) and np.isfinite(hi) and lo < hi and np.isfinite(scale)):
        raise ValueError("uniform_f32 needs finite low < high with a finite width")
    while True:
        res = _uniform_from_words(np.array([rng.next_u32()], np.uint32), lo, scale)[0]
        if res < hi:
            return res


def _uniform_from_words(u: np.ndarray, lo: np.float32, scale: np.float32) -> np.ndarray:
    v12 = (np.uint32(0x3F800000) | (u >> np.uint32(9))).astype(np.uint32).view(np.float32)
    v01 = (v12 - np.float32(1.0)).astype(np.float32)
    return ((v01 * scale).astype(np.float32) + lo).astype(np.float32)


def reference_start_velocities(n: int, seed: int = 0) -> np.ndarray:
    """(n, 3) float32: per agent (gen_range(-0.8..0.8), 0, gen_range(-0.8..0.8)), x drawn before z."""
    lo, hi = np.float32(-0.8), np.float32(0.8)
    scale = np.float32(hi - lo)
    rng = ChaCha8Rng(seed)
    draws = _uniform_from_words(rng.words(2 * n), lo, scale)
    if np.all(draws < hi):  # no redraw: one word per sample
        xz = draws.reshape(n, 2)
    else:  # a redraw shifts every later sample: draw them one by one
        rng = ChaCha8Rng(seed)
        xz = np.array([uniform_f32(rng, lo, hi) for _ in range(2 * n)], np.float32).reshape(n, 2)
    v = np.zeros((n, 3), np.float32)
    v[:, 0] = xz[:, 0]
    v[:, 2] = xz[:, 1]
    return v
