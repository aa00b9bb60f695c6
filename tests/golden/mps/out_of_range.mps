NAME out_of_range
ROWS
 N  OBJ
 L  R1
COLUMNS
    A         OBJ        1.0      R1         1e400
ENDATA
