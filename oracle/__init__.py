"""CPU restatement of Gravity-Sim's force-and-integrate path (test infrastructure only)."""
