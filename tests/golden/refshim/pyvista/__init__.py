"""Empty stand-in: the reference imports pyvista at module top but only
Mesher.to_vtk uses it."""
