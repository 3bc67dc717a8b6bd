"""CPU oracle for the 3D pure-qP VTI loop -- test infrastructure only."""
