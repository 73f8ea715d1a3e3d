"""GPU taggers that the reference's factory resolves as jellyfysh.activator.tagger modules."""
