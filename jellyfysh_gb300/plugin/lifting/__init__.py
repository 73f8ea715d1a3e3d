"""GPU lifting schemes with the reference's class interface (one module per class, as the reference's factory
requires)."""
