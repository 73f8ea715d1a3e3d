"""GPU potentials with the reference's constructor and method signatures (one module per class, as the
reference's factory requires)."""
