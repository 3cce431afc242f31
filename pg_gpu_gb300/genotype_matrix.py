"""Drop-in for the LD subset of pg_gpu.genotype_matrix.GenotypeMatrix.

Holds an (n_individuals x n_variants) int8 dosage matrix (0/1/2, -1 =
missing), its positions and population sample sets (genotype_matrix.py:
15-145); the device copy is a CUDA torch tensor.
"""
from __future__ import annotations

import numpy as np

from . import _lib as L
from . import _ops


def _is_dev(x):
    try:
        import torch
        if isinstance(x, torch.Tensor):
            return x.is_cuda
    except ImportError:
        pass
    return hasattr(x, "__cuda_array_interface__")


class GenotypeMatrix:
    def __init__(self, genotypes, positions, chrom_start=None, chrom_end=None,
                 sample_sets=None, n_total_sites=None, samples=None, accessible_mask=None):
        shape = tuple(genotypes.shape)
        if int(np.prod(shape)) == 0:
            raise ValueError("genotypes cannot be empty")
        if len(positions) == 0:
            raise ValueError("positions cannot be empty")
        if _is_dev(genotypes):
            self._device = "GPU"
            self._genotypes = L.as_device(genotypes, np.int8)
            self._positions = L.as_device(positions)
        else:
            self._device = "CPU"
            self._genotypes = np.asarray(genotypes)
            p = positions
            self._positions = np.asarray(p.cpu().numpy() if hasattr(p, "cpu") else p)
        self.chrom_start = chrom_start
        self.chrom_end = chrom_end
        self._sample_sets = sample_sets
        self.n_total_sites = n_total_sites
        self.samples = samples
        self.accessible_mask = accessible_mask
        self._packed = {}

    @property
    def genotypes(self):
        return self._genotypes

    @genotypes.setter
    def genotypes(self, value):
        self._genotypes = value
        self._packed = {}

    @property
    def positions(self):
        return self._positions

    @positions.setter
    def positions(self, value):
        self._positions = value

    @property
    def device(self):
        return self._device

    @property
    def sample_sets(self):
        if self._sample_sets is None:
            return {"all": list(range(self.num_individuals))}
        return self._sample_sets

    @sample_sets.setter
    def sample_sets(self, sample_sets):
        self._sample_sets = sample_sets
        self._packed = {}

    @property
    def shape(self):
        return tuple(self._genotypes.shape)

    @property
    def num_variants(self):
        return int(self._genotypes.shape[1])

    @property
    def num_individuals(self):
        return int(self._genotypes.shape[0])

    @property
    def has_accessible_mask(self):
        return self.accessible_mask is not None

    def __repr__(self):
        return (f"GenotypeMatrix(shape={self.shape}, device={self._device})")

    def transfer_to_gpu(self):
        if self._device == "CPU":
            self._genotypes = L.as_device(self._genotypes, np.int8)
            self._positions = L.as_device(self._positions)
            self._device = "GPU"

    def transfer_to_cpu(self):
        if self._device == "GPU":
            self._genotypes = self._genotypes.cpu().numpy()
            self._positions = self._positions.cpu().numpy()
            self._device = "CPU"
            self._packed = {}

    def _pos_np(self):
        p = self._positions
        return p.cpu().numpy() if hasattr(p, "cpu") else np.asarray(p)

    @classmethod
    def from_haplotype_matrix(cls, hap_matrix):
        """Pair haplotypes (0,1), (2,3), ... into dosages; a missing haplotype makes
        the dosage missing; sample sets map to individual indices
        (genotype_matrix.py:248-305)."""
        hap = hap_matrix.haplotypes
        n_hap = int(hap.shape[0])
        if n_hap % 2:
            raise ValueError(f"Need even number of haplotypes for diploid conversion, got {n_hap}")
        if _is_dev(hap):
            import torch
            h = L.as_device(hap, np.int8)
            h1, h2 = h[0::2], h[1::2]
            g = (h1.clamp(min=0) + h2.clamp(min=0)).to(torch.int8)
            g[(h1 < 0) | (h2 < 0)] = -1
        else:
            h = np.asarray(hap)
            h1, h2 = h[0::2], h[1::2]
            g = (np.maximum(h1, 0) + np.maximum(h2, 0)).astype(np.int8)
            g[(h1 < 0) | (h2 < 0)] = -1
        sets = None
        if getattr(hap_matrix, "_sample_sets", None) is not None:
            sets = {k: sorted(set(i // 2 for i in v)) for k, v in hap_matrix._sample_sets.items()}
        return cls(g, hap_matrix.positions, hap_matrix.chrom_start, hap_matrix.chrom_end,
                   sample_sets=sets, n_total_sites=getattr(hap_matrix, "n_total_sites", None))

    @classmethod
    def from_vcf(cls, path, include_invariant=False, accessible_bed=None):
        """Alt-allele dosages of a plain or gzipped VCF through the native GT
        reader, kept to the sites whose called alleles are exactly {0, 1}
        (allel's is_biallelic_01); -1 where either allele is missing
        (genotype_matrix.py:343-391)."""
        from .haplotype_matrix import read_vcf_gt
        names, hap, pos = read_vcf_gt(path)
        n = len(names)
        a, b = hap[:n], hap[n:]
        keep = (hap == 0).any(0) & (hap == 1).any(0) & ~(hap > 1).any(0)
        a, b, pos = a[:, keep], b[:, keep], pos[keep]
        g = (a.astype(np.int16) + b).astype(np.int8)
        g[(a < 0) | (b < 0)] = -1
        if g.shape[1] == 0:
            raise ValueError(f"No biallelic variants found in {path}")
        gm = cls(np.ascontiguousarray(g), pos, int(pos[0]), int(pos[-1]), samples=list(names),
                 n_total_sites=g.shape[1] if include_invariant else None)
        if accessible_bed is not None:
            # variants at inaccessible positions are dropped (the reference
            # masks them by the first record's chromosome)
            from .accessible import accessible_variants
            from .haplotype_matrix import vcf_first_chrom
            chrom = vcf_first_chrom(path)
            keep = accessible_variants(pos, accessible_bed, chrom)
            cs, ce = gm.chrom_start, gm.chrom_end
            gm = gm.get_subset(np.nonzero(keep)[0])
            # the per-base denominator: the BED's accessible bases in the range
            from .accessible import accessible_base_count
            gm.chrom_start, gm.chrom_end = cs, ce
            gm.n_total_sites = accessible_base_count(accessible_bed, chrom, cs, ce)
        return gm

    def load_pop_file(self, pop_file, pops=None):
        """Population sample sets from a sample / pop file (genotype_matrix.py:475-504)."""
        if self.samples is None:
            raise ValueError("No sample names stored. Use from_vcf() to load data.")
        pop_map = {}
        with open(pop_file) as f:
            for line in f:
                parts = line.strip().split()
                if len(parts) >= 2 and parts[0] != "sample":
                    pop_map[parts[0]] = parts[1]
        if pops is None:
            pops = sorted(set(pop_map.values()))
        sets = {p: [] for p in pops}
        for i, name in enumerate(self.samples):
            p = pop_map.get(name)
            if p in sets:
                sets[p].append(i)
        self.sample_sets = sets

    def get_subset(self, idx):
        g = self._genotypes[:, idx]
        p = self._positions[idx]
        out = GenotypeMatrix(g, p, self.chrom_start, self.chrom_end,
                             sample_sets=self._sample_sets, samples=self.samples)
        return out

    def apply_biallelic_filter(self):
        """Keep variants whose alt-allele count among called individuals lies
        strictly between 0 and 2 x called, with at least 2 called
        (genotype_matrix.py:506-530)."""
        g = self._genotypes
        if self._device == "GPU":
            import torch
            v = g >= 0
            alt = torch.where(v, g, torch.zeros_like(g)).to(torch.int64).sum(0)
            nv = v.sum(0)
            idx = ((alt > 0) & (alt < 2 * nv) & (nv >= 2)).nonzero().flatten()
        else:
            v = g >= 0
            alt = np.where(v, g, 0).astype(np.int64).sum(0)
            nv = v.sum(0)
            idx = np.where((alt > 0) & (alt < 2 * nv) & (nv >= 2))[0]
        return self.get_subset(idx)

    # --------------------------------------------------------------- packing
    def packed(self, pop=None):
        self.transfer_to_gpu()
        if pop not in self._packed:
            rows = None if pop is None else self.sample_sets[pop]
            self._packed[pop] = _ops.pack_geno(self._genotypes, rows)
        return self._packed[pop]
