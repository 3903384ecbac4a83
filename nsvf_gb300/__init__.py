"""nsvf_gb300: GB300-native (sm_103a) sparse-voxel rendering hot path of NSVF.

Drop-in layers, from the bottom:

* ``nsvf_gb300.ext``       -- the native op module (``fairnr.clib._ext``)
* ``nsvf_gb300.clib``      -- the op API (``fairnr.clib``)
* ``nsvf_gb300.geometry``  -- geometry helpers (``fairnr.data.geometry``)
* ``nsvf_gb300.encoder``   -- ``SparseVoxelEncoder``
* ``nsvf_gb300.renderer``  -- ``VolumeRenderer``

The C ABI is declared in include/nsvf_gb300.h and built by
``python -m nsvf_gb300.build`` into nsvf_gb300/_build/libnsvf_gb300.so.
"""
__version__ = "0.1.0"
