"""``get_normalized_weighting`` as fullrmc calls it
(``Constraints/PairDistributionConstraints.py:487``): element-pair weights
keyed ``"A-B"`` from the number of atoms per element and the elements'
scattering weights, by the definition in fullrmc's documentation
(``PairDistributionConstraints.py:66-86``):

    w_ij = (2 - delta_ij) c_i c_j b_i b_j / (sum_k c_k b_k)^2,  c_i = n_i / N.

The published package's own arithmetic is not available here, so its
values are not pinned; both sides of every comparison use these."""
import itertools

import numpy as np


def get_normalized_weighting(numbers, weights):
    elements = sorted(numbers.keys())
    n = np.array([numbers[e] for e in elements], np.float64)
    b = np.array([weights[e] for e in elements], np.float64)
    c = n / n.sum()
    s = (c * b).sum()
    out = {}
    for i, j in itertools.combinations_with_replacement(range(len(elements)), 2):
        w = c[i] * b[i] * c[j] * b[j] / (s * s)
        if i != j:
            w = 2.0 * w
        out["%s-%s" % (elements[i], elements[j])] = w
    return out
