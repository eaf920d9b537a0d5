"""CPU oracle (test infrastructure only): C restatement of pygetm's Fortran
operators plus a numpy restatement of their Python orchestration."""
