"""acd-alm for GB300: the ALM + APPROX LP solve loop as a CUDA (sm_103a)
C-ABI library, ``libacdalm.so``, behind the reference's alm.h / approx.h /
spmv.h / thread_pool.h interface.

Python users load the library through :mod:`.lib` (ctypes); C users link
``libacdalm.so`` and include ``include/*.h``.  :mod:`.instances` builds the
seeded synthetic workloads.
"""
