"""CPU oracle for the AstroPhot render + Levenberg-Marquardt path.

TEST INFRASTRUCTURE ONLY.  Nothing in the product package imports this
package; only ``tests/``, ``__graft_entry__.smoke()`` and the
``cpu_baseline`` / ``--impl reference`` legs of ``bench.py`` use it, and
there only as the checker or as the timed CPU baseline, never as the thing
being measured or shipped.

The oracle is a float64 numpy restatement of the reference's algorithm
(AstroPhot 0.x, ``astrophot/``), each function citing the reference
file:line it follows.  It is pinned against golden vectors produced by the
reference itself (``tests/golden/make_golden.py`` imports the reference and
records its outputs; ``tests/test_oracle_golden.py`` checks the oracle
against them).
"""

from .render import (  # noqa: F401
    Window,
    Component,
    PSF,
    sample_component,
    sample_group,
    sersic_b,
    sersic_total_flux,
    value_to_rep,
    rep_to_value,
    drep_dvalue,
    moffat_psf,
    gaussian_psf,
)
from .lm import LMOracle, GroupProblem  # noqa: F401
