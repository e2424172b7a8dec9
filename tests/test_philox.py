"""Philox4x32-10 known-answer vectors, the stream layout and the direction math."""

import numpy as np


def test_philox_known_answers(orc):
    # Published known-answer vectors of Philox4x32-10 (Random123 kat_vectors).
    kat = [
        ((0, 0, 0, 0), (0, 0), (0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8)),
        ((0xffffffff,) * 4, (0xffffffff,) * 2, (0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd)),
        ((0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344), (0xa4093822, 0x299f31d0),
         (0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1)),
    ]
    for ctr, key, want in kat:
        assert tuple(int(x) for x in orc.philox(ctr, key)) == want


def test_stream_layout(orc):
    seed, w = 0x1234_5678_9abc_def0, 77
    words = orc.stream_words(seed, w, 12)
    for k in range(12):
        blk = orc.philox((k // 4, 0, w, 0), (seed & 0xffffffff, seed >> 32))
        assert words[k] == blk[k % 4]


def test_sincos_polynomial_accuracy(orc):
    u = (np.arange(0, 1 << 23, 997) + 0.5) / (1 << 23)
    s = np.array([orc.sincos_2pi_f32(float(x)) for x in u])
    ref_s, ref_c = np.sin(2 * np.pi * u), np.cos(2 * np.pi * u)
    assert np.max(np.abs(s[:, 0] - ref_s)) < 4e-7
    assert np.max(np.abs(s[:, 1] - ref_c)) < 4e-7
    # exact quadrant points
    assert orc.sincos_2pi_f32(0.25) == (1.0, 0.0)
    assert orc.sincos_2pi_f32(0.5) == (0.0, -1.0)
