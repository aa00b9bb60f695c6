* comment line, then a blank line

NAME          edge_sections  extra_token
OBJSENSE
    MAX
ROWS
 N  COST
 E  BAL1
 l  CAP2
 G  DEM3
 E  RNG4
 E  RNG5
 G  RNG6
 L  RNG7
 N  SECOND_OBJ
 E  BAL1
 X  ODD8
COLUMNS
    X1        COST       1.5   BAL1       1.0
    X1        CAP2       2.0   DEM3       1e-17
    X1        NOWHERE    9.0   SECOND_OBJ 4.0
    X2        COST      -2.0   CAP2       1.0
    X2        BAL1       0.5   BAL1       0.25
    MARKER                 'MARKER'                 'INTORG'
    X3        COST       3.0   DEM3       1.0
    X3        RNG4       1.0   RNG5       1.0
    MARKER                 'MARKER'                 'INTEND'
    X4        RNG6       1.0   RNG7       1.0
    X4        ODD8       2.0   COST       0.5
    X1        RNG4       -1.0
    X2        DEM3       7.0   DEM3      -7.0
    X5        COST       0.0
FOOBAR
RHS
    RHS1      BAL1       4.0   CAP2      10.0
    DEM3       2.0
    RHS1      COST      12.5
    RHS1      RNG4       1.0   RNG5       2.0
    RHS1      RNG6       3.0   RNG7       4.0
RANGES
    RNG1      RNG4       2.0   RNG5      -3.0
    RNG1      RNG6      -1.5   RNG7      -2.5
BOUNDS
 UP BND       X1         4.0
 LO BND       X2        -1.0
 UP BND       X2         3.0
 FX BND       X3         0.5
 FR BND       X4
 MI BND       X5
 PL BND       X6
 BV BND       X7
 UI BND       X8         9.0
 LI BND       X8         2.0
ENDATA
    X9        COST       1.0
