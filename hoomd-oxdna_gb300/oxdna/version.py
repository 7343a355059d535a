"""Package version."""

version = "1.0.0"
