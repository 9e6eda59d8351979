"""Build recipe and driver of the reference's own Krylov code (test infrastructure only)."""
