"""Import stub for astropy (FITS I/O is not used by the fixture script)."""
