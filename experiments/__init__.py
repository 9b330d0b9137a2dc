"""Measurement drivers cited by the notes and the kernel profiles (not part of
the library): the profiling case (cases.py) and the learned-radius
experiment (rs_experiment.py)."""
