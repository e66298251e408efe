"""CPU oracle for the PNGF direct-binary-search hot path.

TEST INFRASTRUCTURE ONLY. Nothing in the product library imports this
package: only the tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg
of ``bench.py`` use it, and only as the checker / CPU baseline.

Contents:
  * ``geometry``   - Yee-edge numbering, tile edge sets and P
                     (pngf-opt/pngfopt.hpp:86-94, 624-674), the source port
                     (pngfopt.hpp:559-618).
  * ``refalg``     - numpy restatements of the reference optimizer's algebra
                     on C^-1 (``RefState``, pngfopt.hpp:196-367,
                     linalg.hpp:34-85) and of the augmented-matrix (M)
                     algebra the GPU path implements (``MState``).
  * ``synth``      - ctypes binding of synth.c: the synthetic G and NF2FF
                     rows (the stand-in for acmefdfd's G files) that every
                     oracle run and golden log uses.
  * ``magichat``   - MagicHat (pngf-opt/magichat.hpp:32-111): std::mt19937
                     plus libstdc++'s uniform_int_distribution, restated.
  * ``dbs``        - the DBS loop of pngf-opt/main.cpp:338-459, both the
                     reference's mirror-symmetric mode and the single-tile mode.
  * ``port``       - ctypes binding of pngf_port.c, the C restatement used as
                     the timed CPU baseline at full sizes.

Parity pin: the reference itself, compiled here from its own headers by
``oracle/Makefile`` (target ``ref``), produced the golden logs under
``tests/golden/``; the tests check this oracle against them.
"""
