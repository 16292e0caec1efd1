// Reads JSON from stdin with bfs::Json, adds a key, writes it back indented.
#include <iostream>
#include <sstream>

#include "bfs_json.hpp"

int main() {
  std::stringstream ss;
  ss << std::cin.rdbuf();
  bfs::Json j = bfs::Json::parse(ss.str());
  j["added"]["nested"] = std::vector<double>{1.5, 2.0, -3.25e-7};
  j["added"]["count"] = 18446744073709551615ull;
  j["added"]["text"] = "a\"b\\c\n";
  std::cout << j.dump(4);
  return 0;
}
