# members of class 8, attributes of their attributes and hubs
C8 TYPE IN -1
-1 F8 OUT -2
-1 M8 OUT -3
-2 F1 OUT -4
-3 F2 OUT -5
