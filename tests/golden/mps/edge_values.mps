NAME          edge_values
ROWS
 N  OBJ
 L  R1
 G  R2
COLUMNS
    A         OBJ        1.5e+2   R1         -.5
    B         OBJ        +3       R2         0x10
    C         OBJ        2.5abc   R1         1D2
    C         R2         -0.0
RHS
    RHS       R1         inf      R2         -1E-3
BOUNDS
 UP BND       A          1e300
 LO BND       B          -inf
ENDATA
