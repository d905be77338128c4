"""Writes tests/golden/kat.json: known-answer vectors for the gate path.

Every expected value here is derived analytically in this script (closed-form
quantum-gate arithmetic with numpy), not by running the oracle or the
library, so the file pins both. The first entry is the reference's own
state test, src/qubit_backend/circuit.rs:802-837 (H(0), H(1), CNOT(0,1) on
two qubits: every amplitude 1/2; the reference asserts it to 0.01).

Run: python tests/golden/make_golden.py
"""
import json
import math
import os

import numpy as np

H, X, Y, Z, RX, RY, RZ, CNOT = range(8)


def c(z):
    z = complex(z)
    return [z.real, z.imag]


def main():
    s2 = 1.0 / math.sqrt(2.0)
    th = 0.7
    kats = []
    kats.append({"name": "reference_circuit_rs_802_hh_cnot", "n": 2,
                 "gates": [[H, 0, -1, 0, 0.0], [H, 1, -1, 0, 0.0], [CNOT, 1, 0, 0, 0.0]],
                 "amplitudes": [c(0.5)] * 4, "tol": 1e-15})
    kats.append({"name": "rx_pi", "n": 1, "gates": [[RX, 0, -1, 0, math.pi]],
                 "amplitudes": [c(math.cos(math.pi / 2)), c(-1j)], "tol": 1e-15})
    kats.append({"name": "ry_half_pi", "n": 1, "gates": [[RY, 0, -1, 0, math.pi / 2]],
                 "amplitudes": [c(math.cos(math.pi / 4)), c(math.sin(math.pi / 4))], "tol": 1e-15})
    kats.append({"name": "ghz3", "n": 3, "gates": [[H, 0, -1, 0, 0.0], [CNOT, 1, 0, 0, 0.0], [CNOT, 2, 1, 0, 0.0]],
                 "amplitudes": [c(s2)] + [c(0)] * 6 + [c(s2)], "tol": 1e-15})
    kats.append({"name": "h_rz", "n": 1, "gates": [[H, 0, -1, 0, 0.0], [RZ, 0, -1, 0, th]],
                 "amplitudes": [c(s2 * np.exp(-0.5j * th)), c(s2 * np.exp(0.5j * th))], "tol": 1e-15})
    kats.append({"name": "pauli_y_on_qubit1", "n": 2, "gates": [[Y, 1, -1, 0, 0.0]],
                 "amplitudes": [c(0), c(0), c(1j), c(0)], "tol": 0.0})
    kats.append({"name": "x_then_z_phase", "n": 2, "gates": [[X, 0, -1, 0, 0.0], [Z, 0, -1, 0, 0.0]],
                 "amplitudes": [c(0), c(-1), c(0), c(0)], "tol": 0.0})
    kats.append({"name": "cnot_control_above_target", "n": 3,
                 "gates": [[X, 2, -1, 0, 0.0], [CNOT, 0, 2, 0, 0.0]],
                 "amplitudes": [c(0)] * 5 + [c(1)] + [c(0)] * 2, "tol": 0.0})
    kats.append({"name": "observable_gate_skipped", "n": 1,
                 "gates": [[X, 0, -1, 1, 0.0]], "amplitudes": [c(1), c(0)], "tol": 0.0})
    expect = []
    for kind in (RX, RY):
        for t in (0.3, 1.1, 2.9):
            expect.append({"kind": kind, "theta": t, "expect_z": math.cos(t), "d_expect_z": -math.sin(t)})
    sampling = {"probs": [0.25, 0.25, 0.5, 0.0],
                "uniforms": [0.0, 0.1, 0.25, 0.2500001, 0.5, 0.75, 0.999],
                "samples": [2 ** 64 - 1, 0, 0, 1, 1, 2, 2]}
    extract = {"samples": [0, 1, 2, 3, 5], "readout_qubits": [0, 1],
               "values": [[1, 1], [-1, 1], [1, -1], [-1, -1], [-1, 1]]}
    out = {"kats": kats, "expect": expect, "sampling": sampling, "extract": extract}
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "kat.json")
    with open(path, "w") as f:
        json.dump(out, f, indent=1)
    print(f"wrote {path}")


if __name__ == "__main__":
    main()
