"""GB300-native engine for the split-step propagation path of MultimodeNonlinearOptics.

``multimodenonlinearoptics_gb300.nonlinearmedium`` is the drop-in replacement of the
reference's ``nonlinearmedium`` module (import it as ``nonlinearmedium``); the engine
itself is the C ABI library ``libnlm_gb300.so`` built by ``build_ext.build()``.

Host-side front ends under the reference's module names: ``poling`` (poling-pattern generators,
numpy) and ``materials`` (the Sellmeier material decorator, sympy; imported on its own).
"""

__all__ = ["build_ext"]
