"""The reference's start-up random stream (bevy_millions_ball_gb300.chacha):
ChaCha8 seeded by rand_core's seed_from_u64, sampled like rand 0.8's f32
gen_range (src/physics/mod.rs:198-212).

Pinned: the ChaCha block function, against the published ChaCha20 test vector
for the all-zero key and nonce (keystream blocks 0 and 1).  The seeding and the
sampling follow the crates' published algorithms; no run of the reference is
available to pin them."""

import numpy as np

from bevy_millions_ball_gb300 import chacha, scenes, unpack_vfme

# ChaCha20, key = 0, nonce = 0: the first two keystream blocks as little-endian words
ZERO_KEY_BLOCKS = [
    "ade0b876 903df1a0 e56a5d40 28bd8653 b819d2bd 1aed8da0 ccef36a8 c70d778b "
    "7c5941da 8d485751 3fe02477 374ad8b8 f4b8436a 1ca11815 69b687c3 8665eeb2",
    "bee7079f 7a385155 7c97ba98 0d082d73 a0290fcb 6965e348 3e53c612 ed7aee32 "
    "7621b729 434ee69c b03371d5 d539d874 281fed31 45fb0a51 1f0ae1ac 6f4d794b",
]


def test_chacha_block_function_matches_the_published_vector():
    got = chacha.chacha_blocks([0] * 8, 0, 2, rounds=20)
    for b, want in enumerate(ZERO_KEY_BLOCKS):
        assert [f"{w:08x}" for w in got[b]] == want.split()


def test_stream_is_block_ordered_and_resumable():
    a = chacha.ChaCha8Rng(0)
    whole = a.words(100)
    b = chacha.ChaCha8Rng(0)
    parts = np.concatenate([b.words(7), b.words(30), b.words(63)])
    np.testing.assert_array_equal(whole, parts)
    np.testing.assert_array_equal(whole[:32], chacha.chacha_blocks(a.key, 0, 2).reshape(-1))


def test_seed_fill_uses_pcg32_steps():
    seed = chacha.pcg32_seed_bytes(0)
    assert len(seed) == 32 and len(set(seed[i:i + 4] for i in range(0, 32, 4))) == 8
    assert chacha.pcg32_seed_bytes(1) != seed


def test_uniform_f32_single_sample():
    rng = chacha.ChaCha8Rng(0)
    u = int(chacha.ChaCha8Rng(0).words(1)[0])
    x = chacha.uniform_f32(rng, -0.8, 0.8)
    v12 = np.uint32(0x3F800000 | (u >> 9)).view(np.float32)
    want = np.float32(np.float32(np.float32(v12 - np.float32(1)) * np.float32(1.6)) + np.float32(-0.8))
    assert x == want and -0.8 <= x < 0.8


def test_reference_default_scene_uses_the_stream():
    sc = scenes.reference_default()
    v, f, m = unpack_vfme(sc.vfme)
    ref = chacha.reference_start_velocities(sc.n)
    np.testing.assert_array_equal(v, ref.astype(np.float16).astype(np.float32))
    assert np.all(v[:, 1] == 0) and np.all(np.abs(v[:, [0, 2]]) <= 0.8)
    assert np.all(m == 1) and np.all(f == 0)
    assert abs(float(v[:, 0].mean())) < 0.02 and abs(float(v[:, 0].std()) - 0.8 / np.sqrt(3)) < 0.02
