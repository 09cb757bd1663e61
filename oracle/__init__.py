"""ORACLE — test infrastructure only.

CPU restatements of the DIVeR reference algorithms for the rendering hot path,
used as the checker by tests/, by __graft_entry__.smoke() and by bench.py's
CPU-baseline / reference arm.  Nothing in the product package (diver_gb300/)
imports, links or runs anything from here, and nothing here is a fallback for
the CUDA path.

Contents
  dda.c        traversal kernels (dense, masked, octree first hit, 8-hit march)
  mlp_eval.c   the real-time fused decoder (DIVeR32 / DIVeR64)
  build.py     gcc recipe -> oracle/_build/liboracle.so
  native.py    ctypes + numpy wrappers of the C restatements
  integrate.py closed-form segment integral (numpy, float64 or float32)
  torch_ref.py torch-CPU restatement of integrate + DIVeR decoder + render,
               used for reference gradients and the CPU baseline
  ref_kernels.py  builds the reference's own CUDA traversal kernels from its
               sources (only where they are present) and runs them to make
               the traversal fixtures in tests/golden/

Parity pins: traversal against fixtures from the reference's own CUDA
kernels; integrate/decoder/render against fixtures from the reference's own
Python modules (tests/golden/make_golden.py).
"""
