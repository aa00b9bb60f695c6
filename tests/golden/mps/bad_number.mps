NAME bad_number
ROWS
 N  OBJ
 L  R1
COLUMNS
    A         OBJ        abc      R1         1.0
ENDATA
