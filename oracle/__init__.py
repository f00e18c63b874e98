"""CPU oracle of the spatial-cell step: TEST INFRASTRUCTURE ONLY.

Used by tests/, __graft_entry__.smoke() (to check the device step) and by bench.py's
cpu_baseline / reference legs.  The product (spatial_cell_gb300) never imports
it.  Two engines live here:

* ``port`` -- oracle/scport.cpp, a CPU restatement of the reference kernels
  (builds anywhere with g++, also where the reference tree is absent);
* ``ref`` -- oracle/ref_harness.cpp, the reference's own kernel headers
  compiled for the host from the reference tree (only where that tree is
  present), used to pin ``port`` and to generate tests/golden.
"""
