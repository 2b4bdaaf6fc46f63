"""CPU oracle for triangle counting — test infrastructure, never product code."""
