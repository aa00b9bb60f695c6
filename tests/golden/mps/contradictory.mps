NAME contradictory
ROWS
 N  OBJ
 L  R1
COLUMNS
    A         OBJ        1.0      R1         1.0
RHS
    RHS       R1         1.0
BOUNDS
 UP BND       A          -1.0
ENDATA
