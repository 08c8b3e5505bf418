"""The oracle: CPU restatement of the reference DROT loops (test infrastructure only)."""
