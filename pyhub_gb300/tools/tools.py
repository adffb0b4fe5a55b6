"""Helpers with the reference's names (pyhub/tools/tools.py:4-30)."""
import os

import numpy as np


def find_file(directory, filename):
    for root, dirs, files in os.walk(directory):
        if filename in files:
            return os.path.join(root, filename)
    raise FileNotFoundError(f"{filename} not found under {directory}")


def count_bit(n):
    """Number of ones in the bit string n."""
    count = 0
    while n:
        count += 1
        n &= (n - 1)
    return count


def int2str(integer, lengh):
    return str(integer).rjust(lengh, "0")


def fidelity(psi, phi):
    return np.absolute(np.dot(np.conjugate(psi), phi)) ** 2
