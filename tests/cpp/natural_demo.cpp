// Exercises the drop-in `natural` surface of include/natural_gb300.hpp the way
// a user of the original library writes it: products, powers, division,
// remainders, std::format / iostream output and decimal / hex input.  Prints
// one result per line.
#include <iostream>
#include <sstream>

#include "natural_gb300.hpp"

int main(int argc, char** argv) {
  std::cout << std::format("{}\n", pow(natural(2), 65536));
  natural a = pow(natural(3), 4000), b = pow(natural(7), 1500) + 12345;
  natural q = a / b, r = a % b;
  std::cout << std::format("{:x}\n", q) << r << "\n";
  std::cout << ((q * b + r) == a ? "ok" : "BAD") << "\n";
  natural f = factorial(2000);
  std::cout << f << "\n";
  // decimal and hex input (natural.h:121-143, 925-951): round trips of an
  // 84,510-digit power, parsed by the split into halves with GPU products
  const natural p = pow(natural(7), 100000);
  std::istringstream in(std::format("{}", p));
  natural x;
  in >> x;
  natural y;
  y.hex(std::format("{:x}", p));
  std::cout << (x == p ? "dec ok" : "dec BAD") << "\n" << (y == p ? "hex ok" : "hex BAD") << "\n";
  (void)argc;
  (void)argv;
  return 0;
}
