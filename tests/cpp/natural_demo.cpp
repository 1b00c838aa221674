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
  // factorials of 0..40 and a few more on one line (n = 9, 10, 16, 17: some
  // bit of the odd primes' exponents is clear in all of them)
  for (uint64_t n : {0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12, 13, 14, 15, 16, 17, 18, 19, 20, 21, 22, 23, 24, 25, 26,
                     27, 28, 29, 30, 31, 32, 33, 34, 35, 36, 37, 38, 39, 40, 63, 64, 100, 127, 128, 255, 1000})
    std::cout << factorial(n) << " ";
  std::cout << "\n";
  // decimal input of short strings, leading zeros and the empty string
  for (const char* t : {"0", "7", "18446744073709551615", "18446744073709551616", "000123", "",
                        "340282366920938463463374607431768211456"}) {
    natural v;
    v.dec(t);
    std::cout << std::format("{:x}", v) << " ";
  }
  std::cout << "\n";
  (void)argc;
  (void)argv;
  return 0;
}
