// bcmc.js -- the reference's CompressedMarchingCubes shape over the N-API addon
// (bcmc_node.cc): `lruCache.reset()`, the UI's counters as properties, and the
// same async methods (js/compressed_marching_cubes.js:1,366,432,580).
'use strict';
const addon = require('./build/Release/bcmc_node');

class CompressedMarchingCubes {
  constructor(device) {
    this._n = new addon.CompressedMarchingCubes(typeof device === 'number' ? device : 0);
    this.lruCache = {reset: () => this._n.lruCacheReset()};
  }
  async setCompressedVolume(volume, compressionRate, volumeDims, volumeScale) {
    await this._n.setCompressedVolume(volume, compressionRate, volumeDims, volumeScale || [1, 1, 1]);
    this.totalBlocks = this._n.stats().totalBlocks;
  }
  async computeSurface(isovalue, perfTracker) {
    const n = await this._n.computeSurface(isovalue, perfTracker || {});
    Object.assign(this, this._n.stats());
    return n;
  }
  // The vertex buffer's contents (8 B per vertex: packed position, block id);
  // the reference hands the GPUBuffer to its render pass instead.
  copyVertices() { return this._n.copyVertices(); }
  get vertexBufferAddress() { return this._n.vertexBufferAddress(); }
  reportMemoryUse() { return this._n.reportMemoryUse(); }
}

module.exports = {CompressedMarchingCubes};
