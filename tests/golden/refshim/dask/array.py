"""Placeholder for dask.array (the table build is driven block by block instead)."""
