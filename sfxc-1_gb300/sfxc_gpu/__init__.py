"""GB300 (sm_103a) implementation of the SFXC correlator-node hot path.

The CUDA kernels and the C ABI live in libsfxc_gpu.so (sources in ../csrc,
declarations in include/sfxc_gpu.h); this package is the host-side mirror of
the reference's correlator-node task interface plus the synthetic-workload
generator used by the tests and the benchmark.
"""
from . import timebase, synth  # noqa: F401
