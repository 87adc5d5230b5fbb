"""Text outputs in the reference's formats (Files.h:19-79).

saveMatrixComplex writes <name>_r.dat and <name>_i.dat: one line per y, each value
followed by a tab, printed with std::setprecision(20) (the %.20g rendering of the float's
value); saveTensorReal writes <name>_<z>.dat with the stream's default precision (%g).
"""
from __future__ import annotations

import os

import numpy as np


def _fmt20(v: np.ndarray) -> str:
    return "".join(format(float(x), ".20g") + "\t" for x in v) + "\n"


def save_matrix_complex(directory, name, field: np.ndarray):
    f = np.asarray(field, np.complex64)
    for suffix, part in (("_r.dat", f.real), ("_i.dat", f.imag)):
        with open(os.path.join(directory, name + suffix), "w") as fh:
            fh.write("".join(_fmt20(row) for row in part.astype(np.float32)))


def save_tensor_real(directory, name, tensor: np.ndarray):
    t = np.asarray(tensor, np.float32)
    for z in range(t.shape[0]):
        with open(os.path.join(directory, f"{name}_{z}.dat"), "w") as fh:
            fh.write("".join("".join(format(float(x), "g") + "\t" for x in row) + "\n" for row in t[z]))


def load_matrix_complex(directory, name) -> np.ndarray:
    def rd(suffix):
        with open(os.path.join(directory, name + suffix)) as fh:
            return np.array([[float(x) for x in line.rstrip("\n").split("\t") if x != ""] for line in fh], np.float64)
    return (rd("_r.dat").astype(np.float32) + 1j * rd("_i.dat").astype(np.float32)).astype(np.complex64)
