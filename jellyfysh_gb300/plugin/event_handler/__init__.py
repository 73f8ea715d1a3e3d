"""GPU event handlers that the reference's factory resolves as jellyfysh.event_handler modules."""
