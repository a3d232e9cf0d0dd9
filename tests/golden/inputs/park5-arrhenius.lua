-- Park (1993) five-reaction air dissociation/exchange set on a one-temperature gas.
--
-- The rate data are those of Park, C. "Review of Chemical Kinetic Problems of
-- Future NASA Missions, I: Earth Entries", J. Thermophysics and Heat Transfer 7(3), 1993,
-- as used by the five-species subset in examples/lmr/3D/cylinder-larc/rm-park-5sp-2T.inp.
-- That file uses the two-temperature 'Park' form k = A*Tc^n*exp(-C/Tc), Tc = T^s*Tv^(1-s).
-- On a single-temperature gas Tv = T, so Tc = T exactly and the rate is the plain
-- Arrhenius form written here.  No Config{} block: the prep-chem defaults apply
-- (rkf, errTol = 1e-3, maxSubcycles = 10000, maxAttempts = 4, no tight coupling).

Reaction{
    'N2 + M <=> N + N + M',
    fr={'Arrhenius', A=7.0e21, n=-1.60, C=113200.0},
    label='r1',
    efficiencies={['N2']=1.0, ['O2']=1.0, ['NO']=1.0, ['N']=4.2857, ['O']=4.2857},
}

Reaction{
    'O2 + M <=> O + O + M',
    fr={'Arrhenius', A=2.0e21, n=-1.5, C=59500.0},
    label='r2',
    efficiencies={['N2']=1.0, ['O2']=1.0, ['NO']=1.0, ['N']=5.0, ['O']=5.0},
}

Reaction{
    'NO + M <=> N + O + M',
    fr={'Arrhenius', A=5.0e15, n=0.0, C=75500.0},
    label='r3',
    efficiencies={['N2']=1.0, ['O2']=1.0, ['NO']=1.0, ['N']=20.0, ['O']=20.0},
}

Reaction{
    'NO + O <=> O2 + N',
    fr={'Arrhenius', A=8.4e12, n=0.0, C=19450.0},
    label='r4',
}

Reaction{
    'N2 + O <=> NO + N',
    fr={'Arrhenius', A=6.4e17, n=-1.0, C=38400.0},
    label='r5',
}
