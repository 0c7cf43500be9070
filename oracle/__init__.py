"""ORACLE — test infrastructure only: the CPU restatement of the reference render path."""
