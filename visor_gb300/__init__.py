"""GB300-native draw path for the Visor Vulkan ICD."""
