$offlisting
* Minimise the distance to a point outside a ring; `w` is fixed and folds
* into constants; the objective is defined through an inequality.
Variables  u, v, w, objvar;
Equations  e1, e2, e3;

e1..  objvar =G= power(u - 2, 2) + (v + 0.5)**2 + w*u;
e2..  sqr(u) + sqr(v) =L= 4;
e3..  sqr(u) + sqr(v) =G= 1;

u.lo = -3; u.up = 3;
v.lo = -3; v.up = 3;
w.fx = 0.25;

Model m / all /;
Solve m using NLP minimizing objvar;
