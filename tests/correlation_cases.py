"""The pair-correlation cases of tests/golden/correlation.npz (made by
tests/golden/make_golden.py from the reference) and the tests that replay them."""

# pair correlations: system, enumerator (0 radial, 1 linear, 2 layerwise), linear axis,
# Miller indices, function (0 density, 1 S110, 2 S220, 3 S221, 4 axes angle), axis
# (0 primary, 1 secondary, 2 auxiliary), named focal point, max_r, bins
CORRELATIONS = [
    ("hs_small", 0, 0, (0, 0, 1), 0, 0, "o", 4.0, 40),
    ("hs_small", 1, 2, (0, 0, 1), 0, 0, "cm", 2.5, 25),
    ("hs_small", 2, 0, (1, 1, 0), 0, 0, "o", 3.0, 30),
    ("hs_tiny", 0, 0, (0, 0, 1), 0, 0, "o", 3.0, 12),
    ("sc_l2", 0, 0, (0, 0, 1), 0, 0, "o", 5.0, 50),
    ("sc_l2", 0, 0, (0, 0, 1), 2, 0, "end", 5.0, 25),
    ("sc_l2", 1, 1, (0, 0, 1), 1, 0, "beg", 3.0, 30),
    ("sc_l2", 2, 0, (0, 1, 1), 3, 0, "o", 4.0, 20),
    ("sc_l2", 0, 0, (0, 0, 1), 4, 0, "o", 6.0, 1),
    ("sc_l5", 2, 0, (0, 0, 1), 0, 0, "o", 6.0, 60),
    ("sc_tiny", 1, 0, (0, 0, 1), 0, 0, "o", 7.0, 14),
    ("poly_banana", 0, 0, (0, 0, 1), 0, 0, "s0", 5.0, 50),
    ("poly_banana", 0, 0, (0, 0, 1), 1, 2, "o", 5.0, 25),
    ("poly_banana", 2, 0, (1, 0, 0), 2, 1, "s2", 4.0, 20),
    ("poly_dense", 1, 0, (0, 0, 1), 4, 0, "s4", 3.0, 30),
    ("psc_bent", 0, 0, (0, 0, 1), 0, 0, "e1", 4.0, 40),
    ("psc_bent", 2, 0, (0, 1, 0), 0, 0, "o0", 3.0, 30),
]
POLY_AXES = ((0.0, 0.3, 1.0), (1.0, 0.0, 0.2))
NAMED_POINTS = [("sc_l2", "o"), ("sc_l2", "cm"), ("sc_l2", "beg"), ("sc_l2", "end"), ("sc_l5", "beg"),
                ("hs_small", "o"), ("hs_small", "cm"), ("poly_banana", "o"), ("poly_banana", "s0"),
                ("poly_banana", "s4"), ("psc_bent", "o1"), ("psc_bent", "b0"), ("psc_bent", "e1")]
