Variables x, obj;
Equations e;
e.. obj =E= arctan(x);
x.lo = -1; x.up = 1;
Model m / all /;
Solve m using NLP minimizing obj;
