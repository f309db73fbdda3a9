// The host frontier's queue and bound set driven by a script on stdin, one
// operation per line, for a differential check of two implementations of
// include/gpuboscia/concurrent_queue.h (the same source compiled against each):
//   push id parent bound      -> (nothing)
//   pop n cutoff              -> ids popped by pop_batch
//   full n cutoff             -> ids popped by pop_full_batch
//   discard parent            -> (nothing)
//   best cutoff               -> best_bound, size, empty
//   bins bound / berase bound -> ConcurrentBoundSet insert / erase_one
//   bbest cutoff              -> ConcurrentBoundSet best_bound
// Every output line starts with the operation's line number.
#include <cstdio>
#include <iostream>
#include <string>
#include <vector>

#include <gpuboscia/concurrent_queue.h>

int main() {
    ConcurrentQueue q;
    ConcurrentBoundSet bs;
    std::string op;
    int line = 0;
    while (std::cin >> op) {
        ++line;
        if (op == "push") {
            int id, parent;
            double bound;
            std::cin >> id >> parent >> bound;
            Node nd(id, parent, 1, {}, {});
            nd.dual_bound = bound;
            q.push(nd);
        } else if (op == "pop" || op == "full") {
            int n;
            double cutoff;
            std::cin >> n >> cutoff;
            const auto b = op == "pop" ? q.pop_batch(n, cutoff) : q.pop_full_batch(n, cutoff);
            std::printf("%d %s", line, op.c_str());
            for (const auto& nd : b) std::printf(" %d", nd.id);
            std::printf("\n");
        } else if (op == "discard") {
            int parent;
            std::cin >> parent;
            q.discard_children(parent);
        } else if (op == "best") {
            double cutoff;
            std::cin >> cutoff;
            std::printf("%d best %.17g %d %d\n", line, q.best_bound(cutoff), q.size(), q.empty() ? 1 : 0);
        } else if (op == "bins" || op == "berase") {
            double bound;
            std::cin >> bound;
            if (op == "bins") bs.insert(bound);
            else bs.erase_one(bound);
        } else if (op == "bbest") {
            double cutoff;
            std::cin >> cutoff;
            std::printf("%d bbest %.17g\n", line, bs.best_bound(cutoff));
        }
    }
    return 0;
}
