"""Test infrastructure: CPU oracle for the MicMec force/integration path."""
