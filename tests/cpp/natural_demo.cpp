// Exercises the drop-in `natural` surface of include/natural_gb300.hpp the way
// a user of the original library writes it: products, powers, division,
// remainders and std::format / iostream output.  Prints one result per line.
#include <iostream>

#include "natural_gb300.hpp"

int main(int argc, char** argv) {
  std::cout << std::format("{}\n", pow(natural(2), 65536));
  natural a = pow(natural(3), 4000), b = pow(natural(7), 1500) + 12345;
  natural q = a / b, r = a % b;
  std::cout << std::format("{:x}\n", q) << r << "\n";
  std::cout << ((q * b + r) == a ? "ok" : "BAD") << "\n";
  natural f = factorial(2000);
  std::cout << f << "\n";
  (void)argc;
  (void)argv;
  return 0;
}
