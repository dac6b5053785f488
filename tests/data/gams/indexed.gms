Set i / 1*3 /;
Variables x(i), obj;
