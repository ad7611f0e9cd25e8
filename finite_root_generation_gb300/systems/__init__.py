"""System plug-ins: polynomial systems other than Stephenson II, tracked by the same
tracker behind the same C ABI (frg_config.system selects one).

A plug-in is a module here that states its system symbolically (sympy):

  NAME        short name; the C ABI reports it from frg_system_info
  UNKNOWNS    the affine unknowns x (at most 21)
  PARAMS      the parameters q; a task is one value per parameter (complex)
  EQUATIONS   one polynomial in the unknowns per unknown, with coefficients that are
              polynomials in the parameters
  SOLVED      one parameter per equation in which the system is linear: the start
              generation draws the unknowns and the other parameters at random and
              solves this square linear system for these, so the random point is an
              exact root of the start system (the finite-root-generation start, the
              same idea as GenerateStart, frgkinematics.cu:13-136, for Stephenson II)

`gen/gen_plugins.py` turns every module listed in PLUGINS into the CUDA evaluation of
the homogenized system (rows of the homotopy Jacobian and the t column) and a plain-C
copy for the oracle. The order of PLUGINS fixes the system ids: Stephenson II is
system 0 and PLUGINS[k] is system k + 1.
"""
PLUGINS = ["conic2", "burmester5"]
