"""Import stub."""
