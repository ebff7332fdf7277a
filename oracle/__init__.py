"""Oracle (test infrastructure only): CPU restatement and reference harness."""
