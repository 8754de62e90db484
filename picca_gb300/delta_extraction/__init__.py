"""Drop-in delta-extraction plugins (GPU expected-flux classes)."""
