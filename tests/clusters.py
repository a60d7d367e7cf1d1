"""Cluster separation as the reference does it (separate_clusters.cpp:355-459),
for building test inputs: breadth-first components over dynamic-dynamic
broad-phase pairs, then each interaction assigned to the clusters holding
its bodies, static bodies joining the clusters they touch."""
from collections import deque


def separate(pairs, is_static, n_bodies):
    adj = [[] for _ in range(n_bodies)]
    for a, b in pairs:
        if not is_static[a] and not is_static[b]:
            adj[a].append(b)
            adj[b].append(a)
    comp = [-1] * n_bodies
    nc = 0
    for s in range(n_bodies):
        if comp[s] >= 0:
            continue
        comp[s] = nc
        q = deque([s])
        while q:
            u = q.popleft()
            for v in adj[u]:
                if comp[v] < 0:
                    comp[v] = nc
                    q.append(v)
        nc += 1
    parts = [[] for _ in range(nc)]
    for p in range(n_bodies):
        parts[comp[p]].append(p)
    inter = [[] for _ in range(nc)]
    for a, b in pairs:
        a, b = int(a), int(b)
        if is_static[a] and is_static[b]:
            continue
        for c in range(nc):
            a_in, b_in = a in parts[c], b in parts[c]
            if a_in:
                if b_in:
                    inter[c].append((a, b))
                elif is_static[b]:
                    parts[c].append(b)
                    inter[c].append((a, b))
            elif b_in and is_static[a]:
                parts[c].append(a)
                inter[c].append((a, b))
    out = []
    for c in range(nc):
        if any(not is_static[p] for p in parts[c]):
            out.append((parts[c], inter[c]))
    return out
