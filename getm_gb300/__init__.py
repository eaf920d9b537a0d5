"""getm_gb300: GB300-native (sm_103a) implementation of pygetm's split-explicit
time-step operators behind pygetm's operator API.

Host set-up (``domain``, ``workloads``) is importable without a GPU; the
operator modules load the CUDA library ``libgetm_gb300.so`` and raise if it is
missing (there is no CPU fallback)."""

__version__ = "0.1.0"
