"""FP64 oracle for the Gaussian kernel-sum path (TEST INFRASTRUCTURE ONLY).

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg use this
package, and only as the checker / the timed CPU reference. The GPU library never imports it.

Two interchangeable libraries export the same C symbols (``oracle_convolve`` ...):

* ``port`` -- ``oracle/gauss_oracle.c``, a C restatement of ``ExactKernel.cxx`` /
  ``AbstractKernel.cxx``, built by :func:`build_port` (runs on any host, including the GPU machine).
* ``reference`` -- ``oracle/_ref/libref_exactkernel.so``, the reference's own ``ExactKernel``
  compiled from its sources by ``oracle/build_ref.sh``; it exists only where the reference tree
  is present (this container), and pins the port through ``tests/golden``.
"""
from .kernels import (  # noqa: F401
    OracleLib,
    build_port,
    build_reference,
    load,
    port_path,
    reference_path,
    reference_root,
)
