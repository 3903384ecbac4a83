"""CPU oracle for the NSVF sparse-voxel hot path.

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() and
by bench.py's CPU-baseline leg, always to check or to time against, never as
the thing measured or shipped. The product package (nsvf_gb300) never
imports it.

* ``oracle.cpu``       -- ctypes front end of the C restatement (clib_oracle.c)
                          plus numpy float64 restatements of the torch-level
                          parts (trilinear interpolation, compositing, MLP).
* ``oracle.build_ref`` -- recipe that compiles the reference's own kernel
                          bodies and octree builder for the CPU (oracle/_ref/),
                          used only where the reference checkout exists.
* ``oracle.ref_clib``  -- ctypes front end of that build.
* ``oracle.ref_import``-- imports the reference's pure-PyTorch modules with
                          their unavailable dependencies stubbed.
"""
