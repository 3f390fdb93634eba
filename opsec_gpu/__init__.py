"""GB300 engine for the OPSEC Fisher-build path (KL signal matrix, band
projections, Fisher matrix and quadratic estimates) behind a C ABI.

``opsec_gpu.api`` binds the shared library built by ``opsec_gpu.build``;
``opsec_gpu.synth`` makes the seeded synthetic inputs of the benchmarks.
"""
__all__ = ["api", "synth", "build"]
