"""GB300-native DISCO-EB perturbation hot path (package source of ``discoeb_gb300``)."""
