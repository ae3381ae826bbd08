"""Diagnostics: ``python -m autopdex_gb300.diag`` builds and runs the throughput probe
(FP64/FP32 FMA rate, atomic scatter rate, copy bandwidth) on the current GPU."""
