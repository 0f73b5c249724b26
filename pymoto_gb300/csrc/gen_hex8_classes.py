"""Writes hex8_classes.cuh: the entries of the hex8 element stiffness of an isotropic cube element (2 x 2 x 2
Gauss points, any Young's modulus, Poisson ratio and edge length) take 10 values up to a sign that does not
depend on the material: K0[i] = sign[i] * value[cls[i]].  The classes are found by evaluating the element
matrix (pymoto_gb300.element_stiffness, host code of the library) at several Poisson ratios and grouping the
entries that are equal up to a fixed sign at all of them.

    python pymoto_gb300/csrc/gen_hex8_classes.py
"""
import os
import sys

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__)))))
import pymoto_gb300 as pg  # noqa: E402

NUS = (0.05, 0.17, 0.3, 0.41, 0.49)


def classes():
    V = np.stack([pg.element_stiffness(3, poisson_ratio=nu).ravel() for nu in NUS], 1)
    keys, cls, sgn = {}, np.zeros(V.shape[0], int), np.zeros(V.shape[0], int)
    for i, row in enumerate(V):
        s = int(np.sign(row[np.argmax(np.abs(row))]))
        k = tuple(np.round(row * s / np.abs(V).max(), 12))
        cls[i] = keys.setdefault(k, len(keys))
        sgn[i] = s
    return cls, sgn, len(keys)


def main():
    cls, sgn, n = classes()
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "hex8_classes.cuh")
    with open(path, "w") as f:
        f.write("// Generated by gen_hex8_classes.py: value classes and signs of the 576 entries of the hex8 element\n"
                "// stiffness of an isotropic cube element (K0[i] = K0_SIGN[i] * value[K0_CLASS[i]]).\n"
                "#pragma once\n\nnamespace pmg {\n\n")
        f.write(f"constexpr int HEX8_CLASSES = {n};\n")
        for name, arr in (("K0_CLASS", cls), ("K0_SIGN", sgn)):
            f.write(f"__host__ __device__ constexpr signed char {name}[576] = {{\n")
            for r in range(24):
                f.write("    " + ", ".join(f"{int(v)}" for v in arr[r * 24:(r + 1) * 24]) + ",\n")
            f.write("};\n")
        f.write("\n}  // namespace pmg\n")
    print(path, n, "classes")


if __name__ == "__main__":
    main()
