"""Philox4x32-10, the counter-based generator of the performance-mode
collision draws, against the published known-answer vectors of Salmon,
Moraes, Dror and Shaw (SC'11; Random123 kat_vectors, philox4x32 with 10
rounds), and the mapping of pair ranks onto its blocks: pair rank k reads
block (k >> 1, c1) and takes words (x0, x1) for even k, (x2, x3) for odd k,
53 bits as (x0 >> 5) * 2^26 + (x1 >> 6)."""
import numpy as np

KAT = [
    # key (k1:k0), counter (x3:x2, x1:x0) -> x0, x1, x2, x3
    (0x0000000000000000, 0x0000000000000000, 0x0000000000000000,
     (0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8)),
    (0xffffffffffffffff, 0xffffffffffffffff, 0xffffffffffffffff,
     (0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd)),
    (0x299f31d0a4093822, 0x85a308d3243f6a88, 0x0370734413198a2e,
     (0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1)),
]


def test_philox_known_answers(oracle_cr):
    for key, c0, c1, want in KAT:
        assert tuple(int(v) for v in oracle_cr.philox_block(key, c0, c1)) == want


def test_pair_rank_mapping(oracle_cr):
    key, c1 = 0x1234_5678_9abc_def0, (7 << 32) | 123
    ks = np.arange(0, 64, dtype=np.uint64)
    u = oracle_cr.philox_uniform(key, ks, np.full(ks.size, c1, dtype=np.uint64))
    for k in range(64):
        x = [int(v) for v in oracle_cr.philox_block(key, k >> 1, c1)]
        a, b = (x[2], x[3]) if k & 1 else (x[0], x[1])
        bits = (a >> 5) * 2 ** 26 + (b >> 6)
        assert u[k] == bits * 2.0 ** -53
    assert np.all((u >= 0) & (u < 1)) and len(np.unique(u)) == u.size
