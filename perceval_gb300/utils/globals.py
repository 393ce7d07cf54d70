"""Global numeric parameters (perceval/utils/globals.py:30-34)."""

global_params = {
    "min_p": 1e-16,
    "min_complex_component": 1e-6,
    "min_precision_gate": 1e-4,
}
