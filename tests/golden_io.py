"""Loaders for the committed golden fixtures (made by golden/make_golden.py
from the reference's own functions)."""
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    return np.load(os.path.join(GOLDEN, name + ".npz"))
