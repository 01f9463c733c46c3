"""CPU oracle (test infrastructure only): a C restatement of PGMax's BP used as the checker."""
