"""GB300-native field-line tracer and squashing-factor (Q) engine."""
