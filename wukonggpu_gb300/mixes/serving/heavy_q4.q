# members of class 10, their hub's attribute and their own
C10 TYPE IN -1
-1 M2 OUT -2
-2 F3 OUT -3
-1 F4 OUT -4
