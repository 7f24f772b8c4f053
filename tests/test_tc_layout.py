"""The tcgen05 operand layout, checked on the CPU: the byte offset the
kernels store an element (r, k) at (mk_umma_offset, mk_tc.cuh) is the
address the shared-memory descriptor of its K = 16 step describes (start
advanced 256 B a step, leading-dimension offset 128 B between the two core
matrices along K, stride-dimension offset K/8 x 128 B between 8-row
groups), every element lands once, and the instruction descriptor encodes
the shape and types where tcgen05.mma kind::f16 reads them."""
import numpy as np
import pytest


def umma_offset(r, k, K):
    return (((r >> 3) * (K >> 3) + (k >> 3)) << 7) + ((r & 7) << 4) + ((k & 7) << 1)


def described(r, k, K):
    kk, kin = divmod(k, 16)
    start, lbo, sbo = 256 * kk, 128, (K // 8) * 128
    return start + (kin // 8) * lbo + (r // 8) * sbo + (r % 8) * 16 + (kin % 8) * 2


@pytest.mark.parametrize("R,K", [(128, 16), (128, 128), (32, 64), (256, 48)])
def test_store_offsets_are_the_described_addresses(R, K):
    offs = np.array([[umma_offset(r, k, K) for k in range(K)] for r in range(R)])
    desc = np.array([[described(r, k, K) for k in range(K)] for r in range(R)])
    assert np.array_equal(offs, desc)
    assert len(np.unique(offs)) == R * K and offs.min() == 0 and offs.max() == 2 * R * K - 2


def test_instruction_descriptor_fields():
    def idesc(M, N, bf16):
        return (1 << 4) | ((1 if bf16 else 0) << 7) | ((1 if bf16 else 0) << 10) | \
            ((N >> 3) << 17) | ((M >> 4) << 24)
    d = idesc(128, 32, True)
    assert (d >> 4) & 3 == 1                 # FP32 accumulator
    assert (d >> 7) & 7 == 1 and (d >> 10) & 7 == 1
    assert (d >> 15) & 3 == 0                # both operands K-major
    assert (d >> 17) & 63 == 4 and (d >> 24) & 31 == 8
    assert idesc(128, 256, False) >> 17 & 63 == 32
