// Test-infrastructure driver, built only by oracle/Makefile against the reference's own
// looper/union_find.h (compiled in place, -DALPS_INDEP_SOURCE), into oracle/_ref/.
//
// stdin:  <n_initial_nodes> <n_ops> then n_ops tokens: "a" (add a node) or "u i j" (unify i j),
//         then a mode word: "list" or "ids".
// "list": one line per node in the format of the reference's unit test (test/union_find.C:55-61):
//         "node i is root and tree size is w" / "node i's parent is p and its root is r".
// "ids":  the number of clusters, then one id per node after set_id/copy_id
//         (union_find.h:324-343), as used by path_integral.C:645-646.
#include <looper/union_find.h>

#include <iostream>
#include <string>
#include <vector>

int main() {
  int n = 0, m = 0;
  std::cin >> n >> m;
  std::vector<looper::union_find::node> v(n);
  for (int k = 0; k < m; ++k) {
    std::string op;
    std::cin >> op;
    if (op == "a") {
      looper::union_find::add(v);
    } else {
      int i, j;
      std::cin >> i >> j;
      looper::union_find::unify(v, i, j);
    }
  }
  std::string mode;
  std::cin >> mode;
  if (mode == "list") {
    for (int i = 0; i < (int)v.size(); ++i) {
      if (v[i].is_root())
        std::cout << "node " << i << " is root and tree size is " << v[i].weight() << "\n";
      else
        std::cout << "node " << i << "'s parent is " << v[i].parent() << " and its root is "
                  << looper::union_find::root_index(v, i) << "\n";
    }
  } else {
    int nc = looper::union_find::set_id(v, 0, (int)v.size(), 0);
    looper::union_find::copy_id(v, 0, (int)v.size());
    std::cout << nc << "\n";
    for (int i = 0; i < (int)v.size(); ++i) std::cout << v[i].id() << "\n";
  }
  return 0;
}
