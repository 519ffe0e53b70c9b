"""GB300-native (sm_103a) implementation of the zk-torch prover field hot path.

Goldilocks / almost-Goldilocks arithmetic, the multilinear product sumcheck,
Basefold commit/open with Poseidon2 Merkle trees, and the Ajtai commitment,
behind the C ABI of goldilocks-cuda-rs / almost-goldilocks-cuda-rs
(include/goldilocks_cuda_wrapper.h, include/almost_goldilocks_cuda_wrapper.h).
The Python modules are thin host-side mirrors of the reference crates' APIs
over that ABI; every computation runs in the CUDA library.
"""
from . import _native
from .memory import DeviceBuffer, synchronize

P = 0xFFFFFFFF00000001
Q_AGL = 0xFFFFFFFEFFFFFFE1


def lib():
    return _native.lib()


__all__ = ["DeviceBuffer", "synchronize", "lib", "P", "Q_AGL"]
