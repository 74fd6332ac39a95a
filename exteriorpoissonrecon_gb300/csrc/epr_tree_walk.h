// Node order of the reference's tree files: RegularTreeNode::write in its non-serialised form
// (Misha/RegularTree.inl:615-642) writes the root, then, for every node that has children, its 2^dim
// children as one block before the subtrees of those children, child c having offset 2 O + bit d of
// c on axis d.  Shared by the .density.tree and .tree writers.
#pragma once

#include <vector>

namespace epr {

struct TreeNodeKey
{
    int t;     // tree depth (the root is 0)
    int O[4];  // offset at that depth
};

// emit(key, hasChildren) is called for every node in file order and returns false to stop;
// hasChildren(key) says whether a node has children.  Returns false when emit stopped the walk.
template <class HasChildren, class Emit>
bool walk_tree(int dim, HasChildren &&hasChildren, Emit &&emit)
{
    TreeNodeKey root{};
    const bool rootKids = hasChildren(root);
    if (!emit(root, rootKids)) return false;
    std::vector<TreeNodeKey> stack;
    if (rootKids) stack.push_back(root);
    while (!stack.empty())
    {
        const TreeNodeKey p = stack.back();
        stack.pop_back();
        TreeNodeKey child[16];
        bool kids[16];
        for (int c = 0; c < (1 << dim); c++)
        {
            child[c].t = p.t + 1;
            for (int d = 0; d < dim; d++) child[c].O[d] = 2 * p.O[d] + ((c >> d) & 1);
            kids[c] = hasChildren(child[c]);
            if (!emit(child[c], kids[c])) return false;
        }
        for (int c = (1 << dim) - 1; c >= 0; c--)
            if (kids[c]) stack.push_back(child[c]);
    }
    return true;
}

}  // namespace epr
