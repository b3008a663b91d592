"""Reference-compatible geometry pre-processing modules (pre_post/ of the reference)."""
