"""Placeholder: the reference imports pandas at module level only for writers."""
