# members of class 9 through six one-to-one and many-to-one steps
C9 TYPE IN -1
-1 F1 OUT -2
-1 M1 OUT -3
-2 F2 OUT -4
-3 F3 OUT -5
-4 M4 OUT -6
