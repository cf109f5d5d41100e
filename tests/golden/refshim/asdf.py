"""Import stub for asdf."""
__version__ = '3.0.0'
