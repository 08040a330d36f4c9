"""Host check of the tcgen05 operand layout used by bx_gemm.cu (no GPU).

The packer stores (row r, k) of a 128x64 BF16 tile at element
((r/8)*8 + k/8)*64 + (r%8)*8 + k%8.  Each MMA (M=128 or N=128, K=16) reads
through a shared-memory descriptor of the canonical no-swizzle K-major form:
core matrices of 8 rows x 16 bytes, K-adjacent cores LBO = 128 B apart,
8-row groups SBO = 1024 B apart, start advanced by 256 B per K step.  This
test walks both mappings and checks they address the same bytes.
"""
import numpy as np


def tile_off(r, k):
    return (((r >> 3) << 3) + (k >> 3)) * 64 + ((r & 7) << 3) + (k & 7)


def desc_byte(start, lbo, sbo, r, k):
    # canonical layout ((8,m),(8,2)):((16B,SBO),(2B,LBO)) for BF16
    return start + (r % 8) * 16 + (r // 8) * sbo + (k % 8) * 2 + (k // 8) * lbo


def test_packed_tile_matches_descriptor_walk():
    seen = set()
    for kk in range(4):              # four K=16 steps per 64-wide block
        for r in range(128):
            for k in range(16):
                b = desc_byte(kk * 256, 128, 1024, r, k)
                assert b == 2 * tile_off(r, kk * 16 + k)
                seen.add(b)
    assert len(seen) == 128 * 64 and max(seen) == 2 * 128 * 64 - 2


def test_packer_is_a_bijection():
    offs = np.array([tile_off(r, k) for r in range(128) for k in range(64)])
    assert np.array_equal(np.sort(offs), np.arange(128 * 64))


def test_instruction_descriptor_fields():
    # kind::f16: FP32 accumulator (bit 4), BF16 A (bits 7-9 = 1) and B
    # (bits 10-12 = 1), K-major A/B, N>>3 at bits 17-22, M>>4 at bits 24-28
    BM, BN = 128, 128
    idesc = (1 << 4) | (1 << 7) | (1 << 10) | ((BN >> 3) << 17) | ((BM >> 4) << 24)
    assert (idesc >> 17) & 0x3F == 16 and (idesc >> 24) & 0x1F == 8
    assert (idesc >> 15) & 3 == 0        # both operands K-major
