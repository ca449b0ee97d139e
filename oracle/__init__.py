"""The oracle: CPU restatement of the reference's TWMC hot path (test infrastructure only)."""
