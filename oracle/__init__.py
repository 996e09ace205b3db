"""CPU oracle for optika_gb300 -- TEST INFRASTRUCTURE ONLY.

A float64 / complex128 NumPy restatement of the reference's sequential
raytrace (optika, pure Python), step for step, used to check the CUDA path.
Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU
baseline import it; the product never calls it.

Parity status:
* multilayer efficiency -- PINNED against the IMD golden vectors that the
  reference's own tests use (optika/materials/_tests/test_multilayers.py:
  178-287), reduced into ``tests/golden/`` by ``tests/golden/make_golden.py``;
* the trace -- pinned by the reference's known-answer identities (closed
  form intercept on the sag, unit normals with z < 0, vector Snell closed
  form, grazing-hyperboloid vertex sheet, grating deflection of the
  reference's grazing spectrograph test), not by outputs of the reference
  itself, which cannot be imported here (its dependency named_arrays is
  absent).  Semantics that live only in named_arrays (TransformationList
  order, histogram edges, interp clamping, matrix power, secant iterates)
  are restated from their documented behaviour.
"""
