"""Exhaustive checks of the integer identities the pair kernels build on, over every input
their lanes can hold (CPU only; the GPU parity tests check the kernels themselves).

* ext_job.cuh, 8-bit pair cells: M = min(hd + s, hd << 7) stands for the reference's
  M = hd ? hd + s : 0 (sw.rs:363-414) wherever M is used (it only meets max(., 0), E >= 0 and
  F >= 0), for hd in [0, 255] and every int8 score s.
* ext_job.cuh, 16-bit pair cells: M = min(hd + s, 32767 * min(hd, 1)) likewise for hd in
  [0, 32767] with hd + s inside int16 (the 16-bit class rule keeps every DP value below 32768).
* global.cu, 4-bit query codes: (b + (b & 0xf0) * 15) * 0x11 + 0x8080 rebuilds the two prmt
  selector bytes 0x80 | c * 0x11 of a column pair b = c0 | c1 << 4 for every code c < 8.
"""
import numpy as np


def _int8_scores():
    return np.arange(-128, 128, dtype=np.int64)


def test_u8_zero_diagonal_guard():
    hd = np.arange(0, 256, dtype=np.int64)[:, None]
    s = _int8_scores()[None, :]
    m_lane = np.minimum(hd + s, hd << 7)
    assert m_lane.min() >= -32768 and m_lane.max() <= 32767  # one signed 16-bit lane
    m_ref = np.where(hd != 0, hd + s, 0)
    # every use of M goes through max(M, 0), max(M, E >= 0, F >= 0) or max(M - cost, 0)
    assert np.array_equal(np.maximum(m_lane, 0), np.maximum(m_ref, 0))
    for cost in (1, 2, 5, 7, 12, 40):
        assert np.array_equal(np.maximum(m_lane - cost, 0), np.maximum(m_ref - cost, 0))


def test_i16_zero_diagonal_guard():
    hd = np.concatenate([np.arange(0, 600), np.arange(32000, 32768)]).astype(np.int64)[:, None]
    s = _int8_scores()[None, :]
    m_lane = np.minimum(hd + s, 32767 * np.minimum(hd, 1))
    m_ref = np.where(hd != 0, hd + s, 0)
    inside = hd + s <= 32767  # the 16-bit class keeps every DP value below 32768
    got = np.where(inside, np.maximum(m_lane, 0), 0)
    want = np.where(inside, np.maximum(m_ref, 0), 0)
    assert np.array_equal(got, want)


def test_q4_selector_rebuild():
    c0 = np.arange(8, dtype=np.uint32)[:, None]
    c1 = np.arange(8, dtype=np.uint32)[None, :]
    b = c0 | (c1 << 4)
    rebuilt = ((b + (b & 0xF0) * 15) * 0x11 + 0x8080) & 0xFFFFFFFF
    want = (0x80 | c0 * 0x11) | ((0x80 | c1 * 0x11) << 8)
    assert np.array_equal(rebuilt, want)
    assert int(rebuilt.max()) < (1 << 16)  # a prmt selector reads only the low 16 bits
