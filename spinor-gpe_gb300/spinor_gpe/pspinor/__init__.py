"""Problem set-up, propagator, array helpers and result container."""
