"""Python mirror of the reference's ParticleSystem (particleSystem.h:50-218).

Same method names and meanings: ``update()`` advances one timestep and
returns False when no particle is left (particleSystem.cpp:892, 963);
``getArray(POSITION)`` returns an (N, 4) float array; ``reactionList`` and
``reactionOrderInfo`` expose the reaction tables (reaction.h:36-66).  The
presets are the reference's test1/test2/test3 scenarios
(particleSystem.cpp:319-571) in its [-1, 1]^3 world.
"""
from __future__ import annotations

import numpy as np

from . import _lib as L
from .system import System

CONFIG_RANDOM, CONFIG_GRID = 0, 1
POSITION, VELOCITY = 0, 1


class ParticleSystem:
    CONFIG_RANDOM = CONFIG_RANDOM
    CONFIG_GRID = CONFIG_GRID
    POSITION = POSITION
    VELOCITY = VELOCITY

    def __init__(self, numParticles, gridSize=(64, 64, 64), bUseOpenGL=False, preset="test3", seed=1,
                 normals="boxmuller"):
        if bUseOpenGL:
            raise ValueError("headless only: no graphics stack")
        self.preset = preset
        self.m_numParticles = int(numParticles)
        if preset == "test1":
            self.deltaTime, self.systemVolume = 0.1, 10.0
            D = [0.0, 0.001, 0.001]
        elif preset == "test2":
            self.deltaTime, self.systemVolume = 0.001, 90.0
            D = [0.0, 0.05, 0.05, 0.05, 0.05]
        else:
            self.deltaTime, self.systemVolume = 0.01, 90.0
            D = [0.0, 0.3, 0.1]
        g = max(gridSize)
        self.sys = System((-1.0, -1.0, -1.0), (1.0, 1.0, 1.0), dt=self.deltaTime, seed=seed, normals=normals,
                          cell_size=2.0 / g if g else 0.0)
        self.m_hDiffusionCoefficients = np.array(D, np.float32)
        for d in D:
            self.sys.add_species(d)
        if preset == "test1":
            self.sys.add_reaction(1, [1], [1, 1], 10.0)        # A -> 2A
            self.sys.add_reaction(2, [1, 2], [2, 2], 2000.0)   # A + B -> 2B
            self.sys.add_reaction(1, [2], [], 10.0)            # B -> 0
        elif preset == "test2":
            self.sys.add_reaction(2, [1, 2], [3], 0.01)        # E + S -> ES
            back = self.sys.add_reaction(1, [3], [1, 2], 1.0)  # ES -> E + S
            self.sys.set_product_placement(back, L.BD_PP_PGEMMAX, 0.2)
            self.sys.add_reaction(1, [3], [1, 4], 1.0)         # ES -> E + P
        self.sys.finalize()
        self._build_tables()
        self.reset(CONFIG_GRID)

    # reference accessors
    def getNumParticles(self):
        return self.sys.count()

    def getNumTypes(self):
        return len(self.m_hDiffusionCoefficients)

    def getDeltaTime(self):
        return self.deltaTime

    def getSystemVolume(self):
        return self.systemVolume

    def getDiffusionCoefficients(self):
        return self.m_hDiffusionCoefficients

    def getGridSize(self):
        return tuple(int(v) for v in self.sys.grid()[0])

    def getCellSize(self):
        return tuple(float(v) for v in self.sys.grid()[1])

    def getWorldOrigin(self):
        return (-1.0, -1.0, -1.0)

    def getCudaPosVBO(self):
        return self.sys.state_pointer()[0]

    def getCudaTypesVBO(self):
        return None

    def _types(self):
        n = self.m_numParticles
        bound = {"test1": n // 2, "test2": n // 11}.get(self.preset, 3 * (n // 4))
        return np.where(np.arange(n) < bound, 1, 2).astype(np.int32)

    def reset(self, config=CONFIG_GRID):
        n = self.m_numParticles
        rng = np.random.Generator(np.random.Philox(1973))
        if config == CONFIG_GRID:
            s = max(int(np.ceil(n ** (1.0 / 3.0) - 1e-9)), 1)
            idx = np.arange(n)
            c = np.stack([idx % s, (idx // s) % s, idx // (s * s)], 1).astype(np.float32)
            spacing = 2.0 / s
            pos = -1.0 + spacing * (c + 0.5) + (rng.random((n, 3), np.float32) * 2 - 1) * spacing * 0.01
        else:
            pos = -1.0 + 2.0 * rng.random((n, 3), np.float32)
        pos = np.clip(pos, -1.0, 1.0).astype(np.float32)
        self.sys.set_particles(pos, self._types())

    def update(self):
        self.sys.step(1)
        return self.sys.synchronize() == L.BD_OK and self.sys.count() > 0

    def getArray(self, array=POSITION):
        if array != POSITION:
            return None
        pos, sp = self.sys.particles()
        out = np.ones((pos.shape[0], 4), np.float32)
        out[:, :3] = pos
        return out

    def setArray(self, array, data, start, count):
        if array != POSITION:
            return
        pos, sp = self.sys.particles()
        pos[start:start + count] = np.asarray(data, np.float32).reshape(count, -1)[:, :3]
        self.sys.set_particles(pos, sp)

    def dumpGrid(self):
        st = self.sys.cells()
        print("maximum particles per cell = %d" % int(np.max(np.diff(st.astype(np.int64)))))

    def dumpParticles(self, start, count):
        a = self.getArray()
        for p in a[start:start + count]:
            print("pos: (%.4f, %.4f, %.4f, %.4f)" % tuple(p))

    def _build_tables(self):
        R = self.sys.n_reactions
        info = [self.sys.reaction_info(r) for r in range(R)]
        self.reactionList = dict(
            order=[i["order"] for i in info], bindRadiusSquared=[i["bind_radius"] ** 2 for i in info],
            unbindRadius=[i["unbind_radius"] for i in info], geminateProbability=[i["geminate_prob"] for i in info],
            prob=[i["prob"] for i in info], rate=[i["rate"] for i in info], nprod=[i["nprod"] for i in info],
            products=[tuple(i["products"]) for i in info], reactants=[tuple(i["reactants"]) for i in info],
            productPositions=[[i["product_offsets"][0], 0, 0, i["product_offsets"][1], 0, 0] for i in info])
        S = self.getNumTypes()
        self.reactionOrderInfo = []
        for o in range(3):
            count = [0] * S
            for i in info:
                if i["order"] == o and o >= 1:
                    count[i["reactants"][0]] += 1
                    if o == 2:
                        count[i["reactants"][1]] += 1
            idx = [0] * S
            for s in range(1, S):
                idx[s] = idx[s - 1] + count[s - 1]
            l2g = [0] * (idx[-1] + count[-1] if S else 0)
            fill = list(idx)
            for r, i in enumerate(info):
                if i["order"] != o or o == 0:
                    continue
                l2g[fill[i["reactants"][0]]] = r
                fill[i["reactants"][0]] += 1
                if o == 2:
                    l2g[fill[i["reactants"][1]]] = r
                    fill[i["reactants"][1]] += 1
            self.reactionOrderInfo.append(dict(
                order=o, reactionsPerOrder=sum(1 for i in info if i["order"] == o), reactionsPerTypeIdx=idx,
                localToGlobal=l2g, localToGlobalSize=len(l2g), numberOfReactionsPerType=count,
                reactionIndexes=[r for r, i in enumerate(info) if i["order"] == o]))
