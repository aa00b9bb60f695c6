NAME
ROWS
 N obj
 E c1
 L c2
COLUMNS
 x obj 1 c1 1
 y obj 2 c1 1
 y c2 3
RHS
 c1 5 c2 6
RANGES
 c2 2
BOUNDS
 UP x 4
 LO BND y 1
ENDATA
