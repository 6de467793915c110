#!/usr/bin/env python3
"""Extract the reference's golden vectors into tests/golden/reference_golden.json.

The reference (LSQuantumED) is C++/PETSc and cannot be built here, so its
googletest sources and PETSc ``.ref`` dumps are read *as text* and their
known answers are copied into one JSON fixture.  The fixture is committed; this
script is only re-run by hand when the extraction itself changes:

    python tests/golden/make_golden.py /path/to/LSQuantumED

Sections (each entry keeps the reference file it came from):
  basis          sizes / row split / int_basis per rank   tests/unit_tests/basis/*
  basis_throw    (N, mag, np) that must raise              tests/unit_tests/basis/*
  int_basis_ref  int_basis.ref listing                     reference_data/int_basis.ref
  elem_diag      get_elem_diag known answers               tests/unit_tests/get_elem_diag/*
  disorder_elem  get_disorder_elem known answers           tests/unit_tests/get_disorder_elem/*
  coup_elems     get_coup_elems column lists               tests/unit_tests/get_coup_elems/*
  matrices       build_diag / build_off_diag / build_disorder dumps (PETSc %g)
  solver         eigenvalues                               tests/unit_tests/solver/*
  correlation    SzSz / SpSm expectation values            tests/unit_tests/correlation/*
  random         RandomDisorder seeds and h_i              tests/unit_tests/tools_random/*
  dsf            DynStructFactor output files              reference_data/dsf_d0_{1,2}.ref
"""
import json
import os
import re
import sys

LAT_RE = re.compile(r'\b(chain1D|square2D|honeycomb2D)\s+(\w+)\s*\{\s*env\s*(?:,\s*(\d+)\s*,\s*(\d+))?\s*\}')
LTYPE = {'chain1D': 0, 'square2D': 1, 'honeycomb2D': 2}


def read(p):
    with open(p) as f:
        return f.read()


def strip_comments(src):
    src = re.sub(r'/\*.*?\*/', '', src, flags=re.S)
    return re.sub(r'//[^\n]*', '', src)


def num(s):
    """Evaluate a numeric literal or a simple a/b expression."""
    s = s.strip()
    if not re.fullmatch(r'[-+0-9.eE/ ]+', s):
        raise ValueError(s)
    if '/' in s:
        a, b = s.split('/')
        return float(a) / float(b)
    return float(s)


def env_nspins(src):
    m = re.search(r'Environment\s+env\s*\{[^,}]*,[^,}]*,\s*(\d+)\s*,', src)
    return int(m.group(1)) if m else None


def meson_np(mesonfile, exe_stem):
    """np for the mpiexec test that runs <exe_stem>.x."""
    txt = read(mesonfile)
    # explicit per-test blocks:  tmp = get_variable('exec_' + 'name' + 'k') ... '-np', 'n'
    m = re.findall(r"get_variable\('exec_'\s*\+\s*'(\w+)'\s*\+\s*'(\w+)'\)\s*test\([^)]*?'-np',\s*'(\d+)'", txt, re.S)
    for name, k, np_ in m:
        if name + k == exe_stem:
            return int(np_)
    # foreach-style blocks: _cases = [...] ... args: ['-np', 'n'
    for blk in re.finditer(r"_cases\s*=\s*\[([^\]]*)\](.*?)'-np',\s*'(\d+)'", txt, re.S):
        cases = re.findall(r"'(\w+)'", blk.group(1))
        for c in cases:
            if exe_stem.endswith(c):
                return int(blk.group(3))
    return None


class RankWalker:
    """Walk statements and report the mpi_rank context each line sits in."""

    def __init__(self, np_):
        self.np = np_ or 1
        self.chain = []
        self.rank = None

    def feed(self, line):
        m = re.search(r'(else\s+)?if\s*\(\s*[\w.]+\.mpi_rank\s*==\s*(\d+)\s*\)', line)
        if m:
            if not m.group(1):
                self.chain = []
            r = int(m.group(2))
            self.chain.append(r)
            self.rank = [r]
            return
        if re.match(r'\s*(\}\s*)?else\s*\{?\s*$', line) and self.chain:
            self.rank = [r for r in range(self.np) if r not in self.chain]
            return

    def ranks(self):
        return self.rank if self.rank is not None else [0]


def split_tests(src):
    parts = re.split(r'\n(?=TEST(?:_F)?\s*\()', src)
    out = []
    for p in parts:
        m = re.match(r'TEST(?:_F)?\s*\(\s*(\w+)\s*,\s*(\w+)\s*\)', p)
        if m:
            out.append((m.group(1) + '.' + m.group(2), p))
    return out


# ---------------------------------------------------------------------------
def extract_basis(root, G):
    d = os.path.join(root, 'tests/unit_tests/basis')
    for fn in sorted(os.listdir(d)):
        if not fn.endswith('.cpp'):
            continue
        src = strip_comments(read(os.path.join(d, fn)))
        N = env_nspins(src)
        np_ = meson_np(os.path.join(d, 'meson.build'), fn[5:-4])
        vecs = {name: [int(x) for x in re.findall(r'-?\d+', body)]
                for name, body in re.findall(r'std::vector<PetscInt>\s+(\w+)\s*\{([^}]*)\}', src)}
        for m in re.finditer(r'ASSERT_THROW\(\s*Basis\s*\(\s*env\s*,\s*(-?\d+)\s*\)', src):
            G['basis_throw'].append({'N': N, 'mag': int(m.group(1)), 'np': np_, 'src': 'tests/unit_tests/basis/' + fn})
        decls = {v: int(mag) for v, mag in re.findall(r'\bBasis\s+(\w+)\s*\{\s*env\s*,\s*(-?\d+)\s*\}', src)}
        walker = RankWalker(np_)
        recs = {}
        for line in src.split('\n'):
            walker.feed(line)
            for var in decls:
                for field in ('size', 'local_size', 'global_start_index', 'nspins_up', 'total_mag', 'nspins', 'mpi_size'):
                    m = re.search(r'(?:EXPECT|ASSERT)_EQ\(\s*(-?\d+)\s*,\s*%s\.%s\s*\)' % (var, field), line)
                    if m:
                        for r in walker.ranks():
                            recs.setdefault((var, r), {})[field] = int(m.group(1))
                m = re.search(r'EXPECT_EQ\(\s*(\w+)\.at\(i\)\s*,\s*%s\.int_basis\.at\(i\)' % var, line)
                if m and m.group(1) in vecs:
                    for r in walker.ranks():
                        recs.setdefault((var, r), {})['int_basis'] = vecs[m.group(1)]
        for (var, r), rec in sorted(recs.items()):
            rec.update({'N': N, 'mag': decls[var], 'np': np_, 'rank': r, 'src': 'tests/unit_tests/basis/' + fn})
            G['basis'].append(rec)
    # int_basis.ref
    txt = read(os.path.join(root, 'tests/unit_tests/reference_data/int_basis.ref'))
    m = re.search(r'A\{(\d+),(-?\d+)\}', txt)
    G['int_basis_ref'] = {'N': int(m.group(1)), 'mag': int(m.group(2)),
                          'values': [int(v) for v in re.findall(r'int_basis\[\d+\]:\s*(\d+)', txt)],
                          'src': 'tests/unit_tests/reference_data/int_basis.ref'}


def extract_elem_diag(root, G):
    d = os.path.join(root, 'tests/unit_tests/get_elem_diag')
    for fn in sorted(os.listdir(d)):
        if not fn.endswith('.cpp'):
            continue
        src = strip_comments(read(os.path.join(d, fn)))
        N = env_nspins(src)
        for name, body in split_tests(src):
            lats = {v: (LTYPE[t], N, int(a) if a else 1, int(b) if b else N) for t, v, a, b in LAT_RE.findall(body)}
            for m in re.finditer(r'EXPECT_EQ\(\s*(-?\d+)\s*,\s*HamiltHelper::get_elem_diag\(\s*neigh_type::(nnn|nn)\s*,\s*(\d+)\s*,\s*(\d+)\s*,\s*(\w+)\s*\)', body):
                lt = lats[m.group(5)]
                G['elem_diag'].append({'ltype': lt[0], 'N': lt[1], 'lx': lt[2], 'ly': lt[3],
                                       'nt': 0 if m.group(2) == 'nn' else 1, 'state': int(m.group(3)),
                                       'expected': int(m.group(1)), 'src': 'tests/unit_tests/get_elem_diag/' + fn})


def extract_disorder_elem(root, G):
    d = os.path.join(root, 'tests/unit_tests/get_disorder_elem')
    for fn in sorted(os.listdir(d)):
        if not fn.endswith('.cpp'):
            continue
        src = strip_comments(read(os.path.join(d, fn)))
        N = env_nspins(src)
        if 'hi[i] = PetscReal(i)/env.nspins' not in src.replace(' ', '').replace('hi[i]=', 'hi[i] = '):
            pass
        for m in re.finditer(r'EXPECT_NEAR\(\s*([-0-9.eE/ ]+?)\s*,\s*\(double\)HamiltHelper::get_disorder_elem\(\s*(\d+)\s*,\s*(\d+)\s*,\s*hi\s*\)\s*,\s*([0-9.eE-]+)\s*\)', src):
            G['disorder_elem'].append({'N': int(m.group(3)), 'state': int(m.group(2)), 'hi': 'i/N',
                                       'expected': num(m.group(1)), 'tol': float(m.group(4)),
                                       'src': 'tests/unit_tests/get_disorder_elem/' + fn})


def extract_coup_elems(root, G):
    d = os.path.join(root, 'tests/unit_tests/get_coup_elems')
    for fn in sorted(os.listdir(d)):
        if not fn.endswith('.cpp'):
            continue
        src = strip_comments(read(os.path.join(d, fn)))
        N = env_nspins(src)
        np_ = meson_np(os.path.join(d, 'meson.build'), fn[5:-4])
        for name, body in split_tests(src):
            bm = re.search(r'\bBasis\s+b\s*\{\s*env\s*,\s*(-?\d+)\s*\}', body)
            lm = LAT_RE.search(body)
            if not bm or not lm:
                continue
            mag = int(bm.group(1))
            t, _, a, b = lm.groups()
            lat = (LTYPE[t], N, int(a) if a else 1, int(b) if b else N)
            walker = RankWalker(np_)
            cur = None
            for line in body.split('\n'):
                walker.feed(line)
                m = re.search(r'get_coup_elems\(\s*neigh_type::(nnn|nn)\s*,\s*b\s*,\s*(\d+)\s*,', line)
                if m:
                    cur = {'ltype': lat[0], 'N': lat[1], 'lx': lat[2], 'ly': lat[3], 'mag': mag, 'np': np_,
                           'ranks': walker.ranks(), 'nt': 0 if m.group(1) == 'nn' else 1,
                           'index': int(m.group(2)), 'ncol': None, 'cols': {},
                           'src': 'tests/unit_tests/get_coup_elems/%s (%s)' % (fn, name)}
                    G['coup_elems'].append(cur)
                    continue
                if cur is None:
                    continue
                m = re.search(r'ASSERT_EQ\(\s*(\d+)\s*,\s*ncol\s*\)', line)
                if m:
                    cur['ncol'] = int(m.group(1))
                m = re.search(r'EXPECT_EQ\(\s*(-?\d+)\s*,\s*coup_elems\[(\d+)\]\s*\)', line)
                if m:
                    cur['cols'][int(m.group(2))] = int(m.group(1))
    for c in G['coup_elems']:
        c['cols'] = [c['cols'][k] for k in sorted(c['cols'])]


def parse_petsc_vec(txt):
    vals = []
    for line in txt.split('\n'):
        line = line.strip()
        if not line or line.startswith(('Vec Object', 'type:', 'Process')):
            continue
        vals.append(float(line))
    return vals


def parse_petsc_mat(txt):
    rows = {}
    for line in txt.split('\n'):
        m = re.match(r'\s*row (\d+):(.*)', line)
        if m:
            rows[int(m.group(1))] = [[int(c), float(v)] for c, v in re.findall(r'\((\d+),\s*([-0-9.eE+]+)\)', m.group(2))]
    return rows


def extract_matrices(root, G):
    base = os.path.join(root, 'tests/unit_tests')
    for sub in ('build_diag/chain_1d', 'build_diag/square_2d', 'build_diag/honeycomb_2d',
                'build_off_diag/chain_1d', 'build_off_diag/square_2d', 'build_off_diag/honeycomb_2d',
                'build_disorder'):
        d = os.path.join(base, sub)
        for fn in sorted(os.listdir(d)):
            if not fn.endswith('.cpp'):
                continue
            src = strip_comments(read(os.path.join(d, fn)))
            dat = re.search(r'"(\w+)\.dat"', src)
            if not dat:
                continue
            stem = dat.group(1)
            ref = os.path.join(base, 'reference_data', stem + '.ref')
            if not os.path.exists(ref):
                continue
            J = {k: num(v) for k, v in re.findall(r'PetscReal\s+(J1|J2|Delta1|Delta2)\s*=\s*([-0-9.eE]+)\s*;', src)}
            N = env_nspins(src)
            mag = int(re.search(r'\bBasis\s+b\s*\{\s*env\s*,\s*(-?\d+)\s*\}', src).group(1))
            t, _, a, b = LAT_RE.search(src).groups()
            calls = re.findall(r'h\.(build_diag|build_off_diag|build_disorder)\s*\(', src)
            hi = 'i/N' if re.search(r'hi\[i\]\s*=\s*PetscReal\(i\)\s*/\s*env\.nspins', src) else None
            txt = read(ref)
            entry = {'name': stem, 'ltype': LTYPE[t], 'N': N, 'lx': int(a) if a else 1, 'ly': int(b) if b else N,
                     'mag': mag, 'J1': J['J1'], 'D1': J['Delta1'], 'J2': J['J2'], 'D2': J['Delta2'],
                     'calls': calls, 'hi': hi,
                     'src': 'tests/unit_tests/%s/%s + tests/unit_tests/reference_data/%s.ref' % (sub, fn, stem)}
            if 'VecView' in src:
                entry['kind'] = 'diag_vec'
                entry['values'] = parse_petsc_vec(txt)
            else:
                entry['kind'] = 'mat'
                entry['rows'] = {str(k): v for k, v in parse_petsc_mat(txt).items()}
            G['matrices'].append(entry)


def extract_solver(root, G):
    d = os.path.join(root, 'tests/unit_tests/solver')
    for fn in sorted(os.listdir(d)):
        if not fn.endswith('.cpp') or 'init' in fn:
            continue
        src = strip_comments(read(os.path.join(d, fn)))
        Nenv = env_nspins(src)
        for name, body in split_tests(src):
            J = {k: num(v) for k, v in re.findall(r'PetscReal\s+(J1|J2|Delta1|Delta2)\s*=\s*([-0-9.eE]+)\s*;', body)}
            mN = re.search(r'env\.nspins\s*=\s*(\d+)', body)
            N = int(mN.group(1)) if mN else Nenv
            bm = re.search(r'\bBasis\s+b\s*\{\s*env\s*,\s*(-?\d+)\s*\}', body)
            lm = LAT_RE.search(body)
            if not (J and bm and lm):
                continue
            t, _, a, b = lm.groups()
            init = re.search(r'SolverInit\(\s*solver\s*,\s*h\.hamilt\s*,\s*(\d+)\s*\)', body)
            dims = re.search(r'EPSSetDimensions\(\s*solver\s*,\s*(\w+)\s*,\s*(\w+)\s*,\s*(\w+)\s*\)', body)
            nev = int(init.group(1)) if init else 1
            ncv = mpd = None
            if dims:
                nev = int(dims.group(1))
                ncv = None if dims.group(2) == 'PETSC_DECIDE' else int(dims.group(2))
                mpd = None if dims.group(3) == 'PETSC_DECIDE' else int(dims.group(3))
            exp = []
            for m in re.finditer(r'solution\(\s*solver\s*,\s*(\d+)\s*,[^;]*;[^;]*;\s*EXPECT_NEAR\(\s*([-0-9.eE]+)\s*,\s*PetscRealPart\(real_eig\)\s*,\s*([0-9.eE-]+)\)', body):
                exp.append([int(m.group(1)), float(m.group(2)), float(m.group(3))])
            refs = re.findall(r'ref_eigs\[(\d+)\]\s*=\s*([-0-9.eE]+)\s*;', body)
            if refs and not exp:
                # test_solver5: loop over nconv comparing ref_eigs[i]; the 9-element
                # buffer makes ref_eigs[9] an out-of-bounds write, so only 0..8 are kept.
                exp = [[int(i), float(v), 1e-13] for i, v in refs if int(i) < 9]
            if not exp:
                continue
            calls = re.findall(r'h\.(build_diag|build_off_diag|build_disorder)\s*\(', body)
            G['solver'].append({'name': name, 'calls': calls, 'ltype': LTYPE[t], 'N': N, 'lx': int(a) if a else 1,
                                'ly': int(b) if b else N, 'mag': int(bm.group(1)), 'J1': J['J1'], 'D1': J['Delta1'],
                                'J2': J['J2'], 'D2': J['Delta2'], 'nev': nev, 'ncv': ncv, 'mpd': mpd,
                                'expected': exp, 'src': 'tests/unit_tests/solver/' + fn})


def extract_correlation(root, G):
    for sub in ('correlation/SzSz', 'correlation/SpSm'):
        d = os.path.join(root, 'tests/unit_tests', sub)
        for fn in sorted(os.listdir(d)):
            if not fn.endswith('.cpp') or fn.startswith('#'):
                continue
            src = strip_comments(read(os.path.join(d, fn)))
            N = env_nspins(src)
            for name, body in split_tests(src):
                J = {k: num(v) for k, v in re.findall(r'PetscReal\s+(J1|J2|Delta1|Delta2)\s*=\s*([-0-9.eE]+)\s*;', body)}
                bm = re.search(r'\bBasis\s+b\s*\{\s*env\s*,\s*(-?\d+)\s*\}', body)
                lm = LAT_RE.search(body)
                om = re.search(r'\b(SzSz|SpSm|SmSp|SiSj)\s+corr\s*\{', body)
                if not (J and bm and lm and om):
                    continue
                t, _, a, b = lm.groups()
                e0 = re.search(r'EXPECT_NEAR\(\s*([-0-9.eE]+)\s*,\s*PetscRealPart\(real_eig\)', body)
                loop = re.search(r'exp_val\[i\]\s*=\s*corr\.ExpectVal\(\s*env\s*,\s*(\d+)\s*,\s*i\s*(\+\s*1)?\s*,', body)
                off = 1 if loop.group(2) else 0
                vals = [(int(m.group(2)), float(m.group(1)), float(m.group(3))) for m in
                        re.finditer(r'EXPECT_NEAR\(\s*([-0-9.eE]+)\s*,\s*PetscRealPart\(exp_val\[(\d+)\]\)\s*,\s*([0-9.eE-]+)\)', body)]
                G['correlation'].append({'name': name, 'op': om.group(1), 'ltype': LTYPE[t], 'N': N,
                                         'lx': int(a) if a else 1, 'ly': int(b) if b else N, 'mag': int(bm.group(1)),
                                         'J1': J['J1'], 'D1': J['Delta1'], 'J2': J['J2'], 'D2': J['Delta2'],
                                         'E0': float(e0.group(1)) if e0 else None,
                                         'pairs': [[int(loop.group(1)), i + off, v, tol] for i, v, tol in vals],
                                         'src': 'tests/unit_tests/%s/%s' % (sub, fn)})


def extract_random(root, G):
    p = os.path.join(root, 'tests/unit_tests/tools_random/test_tools_random1.cpp')
    src = strip_comments(read(p))
    m = re.search(r'RandomDisorder\s+rd\s*\{\s*(\d+)\s*,\s*PETSC_(TRUE|FALSE)\s*,\s*([-0-9.eE]+)\s*,\s*([-0-9.eE]+)\s*,\s*(\d+)\s*\}', src)
    seeds = {int(i): int(v) for v, i in re.findall(r'EXPECT_EQ\(\s*(\d+)\s*,\s*rd\.srand_seq\[(\d+)\]\s*\)', src)}
    him = re.search(r'rd\.hi_init\(\s*(\d+)\s*\)', src)
    his = {int(i): float(v) for v, i in re.findall(r'EXPECT_NEAR\(\s*([-0-9.eE]+)\s*,\s*rd\.hi\[(\d+)\]', src)}
    G['random'] = {'nspins': int(m.group(1)), 'reprod': m.group(2) == 'TRUE', 'min': float(m.group(3)),
                   'max': float(m.group(4)), 'rep': int(m.group(5)),
                   'seeds': [seeds[k] for k in sorted(seeds)], 'hi_index': int(him.group(1)),
                   'hi': [his[k] for k in sorted(his)], 'tol': 1e-13,
                   'src': 'tests/unit_tests/tools_random/test_tools_random1.cpp'}


def extract_dsf(root, G):
    for stem, test, op in (('dsf_d0_1', 'test_dsf1.cpp', 'Sqz'), ('dsf_d0_2', 'test_dsf2.cpp', 'Sqp')):
        txt = read(os.path.join(root, 'tests/unit_tests/reference_data', stem + '.ref'))
        src = strip_comments(read(os.path.join(root, 'tests/unit_tests/phys', test)))
        J = {k: num(v) for k, v in re.findall(r'PetscReal\s+(J1|J2|Delta1|Delta2)\s*=\s*([-0-9.eE]+)\s*;', src)}
        t, _, a, b = LAT_RE.search(src).groups()
        N = env_nspins(src)
        gs = float(re.search(r'GS:\s*([-0-9.eE]+)', txt).group(1))
        nev = int(re.search(r'nev:\s*(\d+)', txt).group(1))
        spins = []
        cur = None
        for line in txt.split('\n'):
            m = re.match(r'# spin:\s*(\d+)', line)
            if m:
                cur = []
                spins.append(cur)
                continue
            m = re.match(r'\s*([-0-9.eE+]+)\s+([-0-9.eE+]+)\s*$', line)
            if m and cur is not None:
                cur.append([float(m.group(1)), float(m.group(2))])
        G['dsf'].append({'name': stem, 'op': op, 'ltype': LTYPE[t], 'N': N, 'lx': int(a) if a else 1,
                         'ly': int(b) if b else N, 'mag0': 0, 'mag1': 1 if op == 'Sqp' else 0,
                         'J1': J['J1'], 'D1': J['Delta1'], 'J2': J['J2'], 'D2': J['Delta2'],
                         'nev': nev, 'GS': gs, 'spins': spins,
                         'src': 'tests/unit_tests/phys/%s + tests/unit_tests/reference_data/%s.ref' % (test, stem)})


def main():
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get('LSQUANTUMED_REF')
    if not root or not os.path.isdir(root):
        sys.exit('usage: make_golden.py <path to the LSQuantumED source tree>')
    G = {k: [] for k in ('basis', 'basis_throw', 'elem_diag', 'disorder_elem', 'coup_elems', 'matrices',
                         'solver', 'correlation', 'dsf')}
    extract_basis(root, G)
    extract_elem_diag(root, G)
    extract_disorder_elem(root, G)
    extract_coup_elems(root, G)
    extract_matrices(root, G)
    extract_solver(root, G)
    extract_correlation(root, G)
    extract_random(root, G)
    extract_dsf(root, G)
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), 'reference_golden.json')
    with open(out, 'w') as f:
        json.dump(G, f, indent=1)
    for k, v in G.items():
        print('%-14s %s' % (k, len(v) if isinstance(v, list) else 'ok'))


if __name__ == '__main__':
    main()
