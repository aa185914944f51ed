# members of class 7 with two attributes and a hub
C7 TYPE IN -1
-1 F6 OUT -2
-1 M7 OUT -3
-2 F7 OUT -4
