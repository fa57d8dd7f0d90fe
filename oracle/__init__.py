"""Oracle package: CPU restatement of the reference (test infrastructure only)."""
