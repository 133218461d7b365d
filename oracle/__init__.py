"""CPU oracle of the recursive-control-variate gradient step (test
infrastructure only; see oracle.py)."""
