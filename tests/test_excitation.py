"""Product-side command parametrisations against the reference's own samplers (golden vectors)."""
import numpy as np


def test_parametrisations_match_reference(golden):
    from spi_gb300 import excitation as ex
    g = golden("commands")
    idxs = list(g["idxs"])
    nu, steps = int(g["n_updates"]), int(g["steps_per_update"])
    c = ex.expand(ex.constant(g["constant_values"], nu, len(idxs), steps), g["default_command"], idxs)
    np.testing.assert_allclose(c, g["constant_commands"], rtol=1e-6, atol=1e-6)
    p = ex.polynomial(g["polynomial_values"], g["ranges"], idxs, nu, steps, int(g["poly_degree"]))
    np.testing.assert_allclose(ex.expand(p, g["default_command"], idxs), g["polynomial_commands"], rtol=1e-5,
                               atol=1e-6)
    b = ex.bezier(g["bezier_values"], g["ranges"], idxs, nu, steps, int(g["bezier_points"]))
    np.testing.assert_allclose(ex.expand(b, g["default_command"], idxs), g["bezier_commands"], rtol=1e-5, atol=1e-6)
