"""GB300-native wavefront path tracer with the xuxmin/DrawLab scene and plugin surface."""
