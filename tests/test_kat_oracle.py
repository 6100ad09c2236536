"""The reference's known-answer tests (tests/kat_cases.py) against the CPU oracle."""
import pytest

import kat_cases
from oracle import raytrace as O


class OracleRunner:
    def plane_intersect(self, geometry, dir, pos):
        return O.finite_plane_intersect(geometry.pos4d, dir.astype(float), pos.astype(float))

    def cylinder_intersect(self, geometry, dir, pos):
        return O.cylinder_intersect(geometry.pos4d, geometry.coos_limits[0], dir.astype(float),
                                    pos.astype(float))

    def transport(self, d1, d2, pol):
        return O.parallel_transport(d1, d2, pol)

    def trace(self, elements, photons, draws=None):
        out, _ = O.run_sequence(elements, photons, draws or {})
        return out


@pytest.mark.parametrize('case', kat_cases.CASES, ids=lambda c: c.__name__)
def test_known_answer_oracle(case):
    case(OracleRunner())
