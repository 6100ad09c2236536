import numpy as np


def normalized_vector(vec):
    vec = np.asarray(vec, dtype=float)
    return vec / np.sqrt(np.sum(vec * vec))


def vector_norm(vec):
    vec = np.asarray(vec, dtype=float)
    return np.sqrt(np.sum(vec * vec))
