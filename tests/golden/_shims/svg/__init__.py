"""Placeholder package so the reference's transport module imports."""
