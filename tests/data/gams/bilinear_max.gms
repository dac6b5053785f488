* A small bilinear maximisation written for these tests (not from a
* benchmark suite): the objective variable is defined by an =E= equation.
Variables  x, y, z, obj;
Positive Variables x, y;
Integer Variables z;
Equations  def, cap, pair;

def..   obj =E= 3*x*y - sqr(x - 1) + 2*z - 0.5*y*y;
cap..   x + 2*y + z =L= 6;
pair..  x*y =G= 0.5;

x.up = 4; y.up = 3;
z.lo = 0; z.up = 2;

Model m / all /;
Solve m using MINLP maximizing obj;
