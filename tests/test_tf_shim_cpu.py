"""The TensorFlow custom-op shim (quantum_gb300/tf_shim/tfq_gb300_tf_ops.cc)
compiles against stand-in TensorFlow headers and the C ABI header, and
registers the five reference op names with the reference's input lists.
TensorFlow itself is absent here; where it is installed,
quantum_gb300.tf_shim.build builds and loads the real op library."""

import re

from quantum_gb300.tf_shim import build as shim


def test_shim_compiles_against_the_abi():
    shim.syntax_check()


def test_shim_registers_the_reference_ops():
    src = open(shim.SRC).read()
    ops = re.findall(r'REGISTER_OP\("(\w+)"\)', src)
    assert ops == ["TfqSimulateExpectation", "TfqSimulateState", "TfqSimulateSamples",
                   "TfqAdjointGradient", "TfqNoisyExpectation"]
    kernels = re.findall(r'REGISTER_KERNEL_BUILDER\(Name\("(\w+)"\)', src)
    assert sorted(kernels) == sorted(ops)
    # input lists of the reference registrations, in order
    want = {
        "TfqSimulateExpectation": ["programs: string", "symbol_names: string",
                                   "symbol_values: float", "pauli_sums: string"],
        "TfqSimulateState": ["programs: string", "symbol_names: string",
                             "symbol_values: float"],
        "TfqSimulateSamples": ["programs: string", "symbol_names: string",
                               "symbol_values: float", "num_samples: int32"],
        "TfqAdjointGradient": ["programs: string", "symbol_names: string",
                               "symbol_values: float", "pauli_sums: string",
                               "downstream_grads: float"],
        "TfqNoisyExpectation": ["programs: string", "symbol_names: string",
                                "symbol_values: float", "pauli_sums: string",
                                "num_samples: int32"],
    }
    for name, inputs in want.items():
        block = src.split(f'REGISTER_OP("{name}")', 1)[1].split("REGISTER_", 1)[0]
        assert re.findall(r'\.Input\("([^"]+)"\)', block) == inputs
